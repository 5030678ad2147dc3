// ffs_fourier_noalloc: the forward transform of one field (real 3D FFT, 2/3 dealiasing,
// 1/(nx ny nz) scaling, FP64) for callers that cannot allocate device memory.
//
// Who needs it: hosts whose device memory belongs to another allocator or memory pool
// (a framework's caching allocator, an arena sized at start-up: a cudaMalloc of its own
// would go around the pool's accounting and fragment what the pool manages), loops that
// must not allocate once running (cudaMalloc and cudaFree can synchronise the device and
// take an unbounded time), and plug-in hosts that grant a component only the buffers
// they pass in. Such callers hand in their own device buffers for the input and the
// output; everything in between (the twiddle tables and the two intermediate passes)
// lives in one fixed device array declared at file scope below.
//
// Limits and rules (also stated in include/ffs.h):
//   * the scratch array holds FFS_NOALLOC_SCRATCH_BYTES (24 MiB) on every GPU that loads
//     the library, until the process exits; grids whose intermediates do not fit are
//     rejected with FFS_EINVAL (128^3 with the 2/3 rule fits);
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that first
//     call before any stream capture;
//   * each call enqueues four kernels and one memset of the caller's output: a kernel
//     that writes the twiddle tables into the array, then the three transform passes.
//     No host memory is read by the device work;
//   * every call rewrites the twiddles and intermediates in the shared array, so calls
//     whose work overlaps on the GPU (different streams, or different host threads)
//     race on it; order them on one stream or synchronise between them;
//   * no cudaMalloc, cudaFree or allocating library routine is called.
#include <mutex>
#include <string>

#include "ffs_engine.cuh"

#define FFS_NOALLOC_SCRATCH_BYTES (24u << 20)

namespace {

// The scratch array. In host code this name is only a stand-in for the symbol: its
// device address comes from cudaGetSymbolAddress (per device, cached below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[FFS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

}  // namespace

namespace ffsgpu {

void set_global_error(const std::string& msg);

// Variant of k_fwd_z_store: forward z pass, 1/N scaling and dealiasing, written straight
// into the caller's full half spectrum [nz][ny][nx/2+1] (complex128, zeros elsewhere
// were written by a memset before).
template <int TX>
__global__ void __launch_bounds__(FFS_MAXT) k_fwd_z_full(Inst<double> I, cplx<double>* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<double>* s0 = reinterpret_cast<cplx<double>*>(smem_raw);
  cplx<double>* s1 = s0 + srows(I.nz) * TX;
  const int kx0 = blockIdx.x * TX, jc = blockIdx.y;
  const int rowstride = I.NYR * I.KXP;
  const cplx<double>* in = I.wz + (long long)jc * I.KXP + kx0;
  const int y = jc < I.ypos ? jc : I.ny - I.NYR + jc;
  const double sc = I.inv_n;
  auto ld = [&](int l, int z) -> cplx<double> { return in[(long long)z * rowstride + l]; };
  auto st = [&](int l, int z, cplx<double> v) {
    const int kx = kx0 + l;
    if (zcomp(I, z) < 0 || kx >= I.Mx) return;
    out[((long long)z * I.ny + y) * I.nxh + kx] = scl(v, sc);
  };
  fft_lines<-1, TX, double>(I.pz, s0, s1, TX, I.twz, ld, st);
}

// Twiddle tables exp(-2 pi i t / n) of the three axes, written into the scratch array
// on the device: sincospi of the FP64 angle fraction -2t/n, exact at multiples of pi/4.
__global__ void k_noalloc_twiddles(cplx<double>* twx, int nx, cplx<double>* twy, int ny, cplx<double>* twz, int nz) {
  const int total = nx + ny + nz;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    cplx<double>* tw = twx;
    int n = nx, t = g;
    if (t >= nx) { t -= nx; tw = twy; n = ny; if (t >= ny) { t -= ny; tw = twz; n = nz; } }
    double sn, c;
    sincospi(-2.0 * (double)t / (double)n, &sn, &c);
    if ((8 * t) % n == 0) {
      const int o = (8 * t) / n;
      const double r = 0.70710678118654752440;   // sqrt(1/2) rounded to FP64
      const double cs8[8] = {1.0, r, 0.0, -r, -1.0, -r, 0.0, r};
      c = cs8[o];
      sn = -cs8[(o + 6) % 8];
    }
    tw[t].x = c;
    tw[t].y = sn;
  }
}

static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace ffsgpu

namespace {

int fourier_noalloc(const double* phys, double* spec, int32_t nx, int32_t ny, int32_t nz, double lx, double ly,
                    double lz, double cutoff, void* stream) {
  using namespace ffsgpu;
  using Eng = Engine<double>;
  auto fail = [](int code, const std::string& m) { set_global_error(m); return code; };
  if (!phys || !spec) return fail(FFS_EINVAL, "ffs_fourier_noalloc: NULL device pointer");
  if (!(lx > 0 && ly > 0 && lz > 0) || !(cutoff > 0 && cutoff <= 1.0))
    return fail(FFS_EINVAL, "ffs_fourier_noalloc: domain sizes must be positive and cutoff in (0, 1]");
  Inst<double> I;
  memset(&I, 0, sizeof(I));
  if (!make_plan(nx, I.px) || !make_plan(ny, I.py) || !make_plan(nz, I.pz))
    return fail(FFS_EUNSUPPORTED, "ffs_fourier_noalloc: unsupported grid size");
  constexpr int TXN = 4;   // kx lines per CTA (FP64)
  if (TXN * std::max(I.py.tpl, I.pz.tpl) > 512 || 2 * LYZ_IO * I.px.tpl > 512 || ((long long)ny * nz) % LYZ_IO)
    return fail(FFS_EUNSUPPORTED, "ffs_fourier_noalloc: unsupported grid size");
  int xp, xc, yp, yc, zp, zc;
  Eng::retained(nx, lx, cutoff, true, xp, xc);
  Eng::retained(ny, ly, cutoff, false, yp, yc);
  Eng::retained(nz, lz, cutoff, false, zp, zc);
  I.nx = nx; I.ny = ny; I.nz = nz; I.nxh = nx / 2 + 1;
  I.lx = lx; I.ly = ly; I.lz = lz;
  I.Mx = xc; I.KXP = ((xc + 7) / 8) * 8;
  I.ypos = yp; I.NYR = yc; I.zpos = zp; I.NZR = zc;
  I.inv_n = 1.0 / ((double)nx * (double)ny * (double)nz);
  I.wys = (long long)nz * ny * I.KXP;
  I.wzs = (long long)nz * I.NYR * I.KXP;
  // scratch layout: twiddles x, y, z | wy (one field) | wz (one field)
  const size_t cb = sizeof(cplx<double>);
  const size_t o_twy = up256(nx * cb), o_twz = o_twy + up256(ny * cb), o_wy = o_twz + up256(nz * cb);
  const size_t o_wz = o_wy + up256((size_t)I.wys * cb), need = o_wz + up256((size_t)I.wzs * cb);
  if (need > FFS_NOALLOC_SCRATCH_BYTES)
    return fail(FFS_EINVAL, "ffs_fourier_noalloc: grid " + std::to_string(nx) + "x" + std::to_string(ny) + "x" +
                                std::to_string(nz) + " needs " + std::to_string(need) +
                                " bytes of scratch; the static buffer holds " +
                                std::to_string(FFS_NOALLOC_SCRATCH_BYTES) + " bytes");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(FFS_ECUDA, "ffs_fourier_noalloc: no usable current CUDA device");
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);   // device `dev` is current
      if (e != cudaSuccess) return fail(FFS_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  I.twx = reinterpret_cast<cplx<double>*>(base);
  I.twy = reinterpret_cast<cplx<double>*>(base + o_twy);
  I.twz = reinterpret_cast<cplx<double>*>(base + o_twz);
  I.wy = reinterpret_cast<cplx<double>*>(base + o_wy);
  I.wz = reinterpret_cast<cplx<double>*>(base + o_wz);
  I.phys = const_cast<double*>(phys);
  const int ntw = nx + ny + nz;
  k_noalloc_twiddles<<<(ntw + 255) / 256, 256, 0, s>>>(reinterpret_cast<cplx<double>*>(base), nx,
                                                      reinterpret_cast<cplx<double>*>(base + o_twy), ny,
                                                      reinterpret_cast<cplx<double>*>(base + o_twz), nz);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemsetAsync(spec, 0, (size_t)nz * ny * I.nxh * cb, s);
  if (e != cudaSuccess) return fail(FFS_ECUDA, std::string("ffs_fourier_noalloc: ") + cudaGetErrorString(e));
  const size_t io = cb * (size_t)srows(nx) * 2 * (2 * LYZ_IO + 1);
  const size_t sy = (size_t)TXN * srows(ny) * cb * (I.py.np >= 3 ? 2 : 1);
  const size_t sz = (size_t)TXN * srows(nz) * cb * (I.pz.np >= 3 ? 2 : 1);
  if (io > 48 * 1024 || sy > 48 * 1024 || sz > 48 * 1024)
    return fail(FFS_EUNSUPPORTED, "ffs_fourier_noalloc: grid size needs more shared memory than this path uses");
  FieldList F{};
  F.n = 1;
  F.code[0] = R_NX;
  F.slot[0] = 0;
  k_phys_fwd_x<double><<<ny * nz / LYZ_IO, round32(2 * LYZ_IO * I.px.tpl), io, s>>>(I, 1, 0);
  k_fwd_y<double, TXN><<<dim3(1, I.KXP / TXN, nz), round32(TXN * I.py.tpl), sy, s>>>(I, F);
  k_fwd_z_full<TXN><<<dim3(I.KXP / TXN, I.NYR), round32(TXN * I.pz.tpl), sz, s>>>(I, reinterpret_cast<cplx<double>*>(spec));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FFS_ECUDA, std::string("ffs_fourier_noalloc launch: ") + cudaGetErrorString(e));
  return FFS_OK;
}

}  // namespace

// No exception crosses the C ABI: std::string work above can throw (bad_alloc).
extern "C" int ffs_fourier_noalloc(const double* phys, double* spec, int32_t nx, int32_t ny, int32_t nz, double lx,
                                   double ly, double lz, double cutoff, void* stream) {
  try {
    return fourier_noalloc(phys, spec, nx, ny, nz, lx, ly, lz, cutoff, stream);
  } catch (const std::exception& ex) {
    ffsgpu::set_global_error(std::string("ffs_fourier_noalloc: internal error: ") + ex.what());
  } catch (...) {
    ffsgpu::set_global_error("ffs_fourier_noalloc: internal error");
  }
  return FFS_EINVAL;
}
