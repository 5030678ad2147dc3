"""Server C ABI on CPU: the ctypes mirrors have the C layout of include/ffs.h (checked by
compiling a probe against the header with gcc), defaults, and a clean failure without a
GPU."""
import ctypes
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

STRUCTS = {
    "ffs_params": "FFSParams",
    "ffs_server_cfg": "FFSServerCfg",
    "ffs_request": "FFSRequest",
    "ffs_result": "FFSResult",
    "ffs_server_info": "FFSServerInfo",
}


def test_struct_layouts_match_header(pkg, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ffs.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in getattr(lib, pyname)._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            s, f, v = line.split()
            got[(s, f)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(lib, pyname)
        assert ctypes.sizeof(cls) == got[(cname, "size")], cname
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == got[(cname, fname)], (cname, fname)


def test_server_defaults(pkg):
    from importlib import import_module
    lib = import_module(pkg.__name__ + "._lib")
    c = lib.FFSServerCfg()
    assert pkg.load().ffs_server_default(ctypes.byref(c)) == 0
    assert c.memory_budget == 120 << 30 and c.max_n == 128 and c.max_active > 0


def test_server_create_without_gpu_fails_cleanly(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    code = (
        "import sys, ctypes; sys.path.insert(0, %r)\n"
        "import __graft_entry__ as ge\n"
        "pkg = ge.load_package(); from ffs_gb300 import _lib\n"
        "L = pkg.load(); c = _lib.FFSServerCfg(); L.ffs_server_default(ctypes.byref(c))\n"
        "h = ctypes.c_void_p(); rc = L.ffs_server_create(ctypes.byref(c), ctypes.byref(h))\n"
        "print(rc, L.ffs_server_last_error(None).decode())\n"
    ) % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rc, msg = r.stdout.strip().split(" ", 1)
    assert int(rc) < 0 and msg
