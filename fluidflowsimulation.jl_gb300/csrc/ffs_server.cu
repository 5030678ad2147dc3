// Batched serving: many independent FP32 simulations on one GPU, advanced together by
// one CUDA graph of batched kernels (ffs_batch.cuh). C ABI in include/ffs.h.
//
// Host side:
//   submit()  -> request queue (fields copied)
//   thread    -> admit while the memory budget and max_active allow: a pooled engine of
//                the same grid and model is repurposed, else a new one is created; its
//                set_fields + initialize! run on the engine's own stream
//             -> rebuild the work tables when the membership changed (pinned staging,
//                stream-ordered upload before the next replay)
//             -> replay the graph: every admitted simulation takes one step
//             -> simulations that reached nt leave the tables; after the next replay has
//                been enqueued, their results are read on their own streams (ordered by
//                an event after their last step) and the engine returns to the pool
//   start     -> with cfg.autotune, each size class's passes are timed in every kernel
//                form on probe simulations and the fastest form per pass is kept; the
//                work tables are cut in the tiles of the chosen forms
//             -> every kHealthEvery replays a one-CTA kernel copies each simulation's
//                error flag (non-finite value seen by its update) to pinned host memory;
//                the host reads the copy one interval later and retires a diverged
//                simulation at once with FFS_ENAN, freeing its slot; cancelled requests
//                (ffs_cancel) leave the queue or the batch the same way
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ffs_batch.cuh"
#include "ffs_engine.h"

namespace ffsgpu {

namespace {

using BI = BatchInst<float>;
constexpr int TXB = BATCH_TX, LYZB = BATCH_LYZ;

struct Job {
  uint64_t id = 0;
  ffs_params p{};
  int64_t nt = 0;
  int keep_fields = 0;
  std::vector<double> u;   // initial fields, 3 * N
  double t_submit = -1, t_admit = -1, t_done = -1;
  int status = FFS_QUEUED;
  bool cancel = false;     // ffs_cancel asked for it while pending or running
  std::string err;
  std::vector<double> stats;
  int ncols = 0;
  std::vector<double> fields;
  int64_t iteration = 0;
  double time = 0, dt = 0;
};

struct Slot {
  std::unique_ptr<EngineBase> eng;
  ffs_params p{};          // parameters the buffers were made for
  int64_t bytes = 0;
  std::shared_ptr<Job> job;   // null: idle, in the pool
  bool retiring = false;
  int64_t done = 0;        // batched steps taken by the current job
  int64_t it0 = 0;         // iteration at admission
  int early = 0;           // FFS_ENAN / FFS_ECANCELED: leaves the batch before nt
  BatchGeom g{};
};

// Error flags of the simulations in the batch (DevState::err), one per slot, gathered
// from the finalize tables (one entry per simulation) so that only live parameter
// blocks are read.
__global__ void k_batch_health(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ T,
                               unsigned* __restrict__ out) {
  for (int c = 0; c < BATCH_NCLASS; ++c) {
    const int n = T->n[c][BP_FIN];
    for (int w = threadIdx.x; w < n; w += blockDim.x) {
      const int k = T->tab[c][BP_FIN][w].inst;
      out[k] = B[k].I.st->err;
    }
  }
}
constexpr int kHealthEvery = 8;   // replays between two health snapshots

// plan threads per line (n / largest radix) and pass count, as make_plan builds them
void plan_shape(int n, int& tpl, int& np) {
  switch (n) {
    case 8: tpl = 1; np = 1; return;
    case 16: tpl = 1; np = 1; return;
    case 32: tpl = 4; np = 2; return;
    case 48: tpl = 12; np = 3; return;
    case 64: tpl = 8; np = 2; return;
    case 96: tpl = 12; np = 3; return;
    case 128: tpl = 8; np = 2; return;
    default: tpl = 0; np = 0; return;
  }
}
const int kSizes[] = {8, 16, 32, 48, 64, 96, 128};

inline int r32(int x) { return ((x + 31) / 32) * 32; }

// Work items of one pass of one simulation (k: its parameter block), in tiles of `tile`
// kx lines (y/z passes) or (y,z) lines (x passes).
void append_items(int ph, int tile, const BatchGeom& g, int k, std::vector<WorkItem>& v) {
  const int kt = g.kxp / tile;
  switch (ph) {
    case BP_INV_Z:
      for (int f = 0; f < g.nin; ++f)
        for (int t = 0; t < kt; ++t)
          for (int jc = 0; jc < g.nyr; ++jc) v.push_back({k, f, t, jc});
      break;
    case BP_INV_Y:
      for (int f = 0; f < g.nin; ++f)
        for (int t = 0; t < kt; ++t)
          for (int z = 0; z < g.nz; ++z) v.push_back({k, f, t, z});
      break;
    case BP_X:
    case BP_X_LES:
      for (int b = 0; b < g.ny * g.nz / tile; ++b) v.push_back({k, b, 0, 0});
      break;
    case BP_FWD_Y:
      for (int f = 0; f < g.nout; ++f)
        for (int t = 0; t < kt; ++t)
          for (int z = 0; z < g.nz; ++z) v.push_back({k, f, t, z});
      break;
    case BP_FWD_Z:
      for (int t = 0; t < kt; ++t)
        for (int jc = 0; jc < g.nyr; ++jc) v.push_back({k, t, jc, 0});
      break;
    default:
      break;
  }
}

// size-class tuning results of this process: (device, side, max_active) -> forms, report
struct ClassTune { int form[BP_COUNT]; std::string report; };
std::mutex& class_tune_mu() { static std::mutex m; return m; }
std::map<std::string, ClassTune>& class_tune_cache() { static std::map<std::string, ClassTune> c; return c; }

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

class Server {
 public:
  ffs_server_cfg cfg{};
  std::string err;           // last error of an API call (guarded by mu)
  std::string terr;          // last CUDA error seen by the serving thread
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Job>> queue;            // submitted, not yet admitted
  std::map<uint64_t, std::shared_ptr<Job>> jobs;     // all known requests
  uint64_t next_id = 1;
  bool stop = false;
  bool paused = false;        // admission held (ffs_server_pause)
  std::thread th;
  std::chrono::steady_clock::time_point t0;
  std::string fatal;          // error that stopped the serving thread
  // statistics (guarded by mu)
  ffs_server_info info{};

  // serving-thread state
  cudaStream_t S = nullptr;
  BI* d_inst = nullptr;
  BI* h_inst = nullptr;       // pinned mirror
  BatchTables* d_tab = nullptr;
  BatchTables* h_tab = nullptr;   // pinned
  WorkItem* h_items[2] = {nullptr, nullptr};   // pinned staging, double-buffered
  size_t h_cap[2] = {0, 0};
  cudaEvent_t h_ev[2] = {nullptr, nullptr};
  int h_cur = 0;
  WorkItem* d_items = nullptr;
  size_t d_cap = 0;
  std::vector<Slot> slots;
  int64_t bytes_in_use = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int grid[BP_COUNT] = {0};
  int block[BP_COUNT] = {0};
  size_t smem[BP_COUNT] = {0};
  ClassOps cls[BATCH_NCLASS] = {};          // size classes 1..: compile-time shapes
  ClassLaunch cl[BATCH_NCLASS] = {};
  cudaStream_t cs[BATCH_NCLASS] = {};       // one branch of the step graph per class
  cudaEvent_t cev[BATCH_NCLASS + 1] = {};   // fork / join events of the capture
  std::vector<cudaEvent_t> ev_pool;
  unsigned* d_health = nullptr;             // [max_active] error flags of the last snapshot
  unsigned* h_health = nullptr;             // pinned copy
  cudaEvent_t health_ev = nullptr;
  std::string tune_report;                  // forms picked per size class and the timings
  std::vector<uint64_t> health_job;         // job id each slot held when the snapshot was taken
  bool health_pending = false;
  int64_t health_at = 0;                    // batch step of the pending snapshot

  ~Server() { shutdown(); }

  int start(const ffs_server_cfg& c) {
    cfg = c;
    if (cfg.max_n <= 0 || cfg.max_n > 128) { err = "max_n must be in 1..128"; return FFS_EINVAL; }
    if (cfg.max_active <= 0) { err = "max_active must be positive"; return FFS_EINVAL; }
    if (cfg.memory_budget <= 0) { err = "memory_budget must be positive"; return FFS_EINVAL; }
    if (cfg.class_forms < 0 || cfg.class_forms > 2) { err = "class_forms must be 0, 1 or 2"; return FFS_EINVAL; }
    t0 = std::chrono::steady_clock::now();
    int rc = setup();
    if (rc) {
      if (err.empty()) err = terr;
      release_gpu();
      return rc;
    }
    th = std::thread([this] { loop(); });
    return 0;
  }

#define SV_CK(call)                                                            \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      terr = std::string(#call) + ": " + cudaGetErrorString(e_);               \
      return FFS_ECUDA;                                                        \
    }                                                                          \
  } while (0)

  // per-kernel limit shared by every server in the process: only ever raised
  template <typename K> int attr(K k, size_t bytes) {
    static std::mutex amu;
    std::lock_guard<std::mutex> g(amu);
    cudaFuncAttributes fa;
    SV_CK(cudaFuncGetAttributes(&fa, k));
    if ((int)bytes > fa.maxDynamicSharedSizeBytes)
      SV_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return 0;
  }
  template <typename K> int occupancy(K k, int ph) {
    int nb = 0, sms = 0;
    SV_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block[ph], smem[ph]));
    SV_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
    if (nb < 1) { terr = "batched kernel does not fit on an SM"; return FFS_EUNSUPPORTED; }
    grid[ph] = nb * sms;
    return 0;
  }

  // launch shapes: the largest over the grid sides the server accepts
  int setup() {
    SV_CK(cudaSetDevice(cfg.device));
    SV_CK(cudaStreamCreateWithFlags(&S, cudaStreamNonBlocking));
    const size_t cb = sizeof(cplx<float>);
    int tplmax = 1;
    size_t s_yz = 0, s_x = 0, s_xl = 0, s_zu = 0;
    for (int n : kSizes) {
      if (n > cfg.max_n) continue;
      int tpl, np;
      plan_shape(n, tpl, np);
      tplmax = std::max(tplmax, tpl);
      const int nb = np >= 3 ? 2 : 1;
      s_yz = std::max(s_yz, (size_t)TXB * srows(n) * cb * nb);
      const size_t mxp = (size_t)(n / 2 + 1) | 1;
      for (int les = 0; les < 2; ++les) {
        const int nin = les ? 11 : 6, pin = (nin + 1) / 2, lin = pin * LYZB;
        const size_t xs = cb * ((size_t)srows(n) * (lin + 1) + std::max((size_t)nin * LYZB * mxp, (size_t)srows(n) * (lin + 1)));
        if (les) s_xl = std::max(s_xl, xs); else s_x = std::max(s_x, xs);
        s_zu = std::max(s_zu, cb * ((size_t)3 * TXB * srows(n) * nb + (size_t)(les ? 4 : 0) * n * TXB));
      }
    }
    block[BP_INV_Z] = block[BP_INV_Y] = block[BP_FWD_Y] = r32(TXB * tplmax);
    smem[BP_INV_Z] = smem[BP_INV_Y] = smem[BP_FWD_Y] = s_yz;
    block[BP_X] = r32(3 * LYZB * tplmax); smem[BP_X] = s_x;
    block[BP_X_LES] = r32(6 * LYZB * tplmax); smem[BP_X_LES] = s_xl;
    block[BP_FWD_Z] = r32(3 * TXB * tplmax); smem[BP_FWD_Z] = s_zu;
    block[BP_SCALAR] = 256; block[BP_TABLE] = 256; block[BP_STATS] = 256; block[BP_UPDATE] = 256;
    block[BP_FIN] = 1024;
    int rc;
    if ((rc = attr(kb_inv_z<float, TXB>, s_yz))) return rc;
    if ((rc = attr(kb_inv_y<float, TXB>, s_yz))) return rc;
    if ((rc = attr(kb_fwd_y<float, TXB>, s_yz))) return rc;
    if ((rc = attr(kb_x<float, false, LYZB>, s_x))) return rc;
    if ((rc = attr(kb_x<float, true, LYZB>, s_xl))) return rc;
    if ((rc = attr(kb_fwd_z<float, TXB>, s_zu))) return rc;
    if ((rc = occupancy(kb_inv_z<float, TXB>, BP_INV_Z))) return rc;
    if ((rc = occupancy(kb_inv_y<float, TXB>, BP_INV_Y))) return rc;
    if ((rc = occupancy(kb_x<float, false, LYZB>, BP_X))) return rc;
    if ((rc = occupancy(kb_x<float, true, LYZB>, BP_X_LES))) return rc;
    if ((rc = occupancy(kb_fwd_y<float, TXB>, BP_FWD_Y))) return rc;
    if ((rc = occupancy(kb_scalar<float>, BP_SCALAR))) return rc;
    if ((rc = occupancy(kb_table<float>, BP_TABLE))) return rc;
    if ((rc = occupancy(kb_fwd_z<float, TXB>, BP_FWD_Z))) return rc;
    if ((rc = occupancy(kb_stats<float>, BP_STATS))) return rc;
    if ((rc = occupancy(kb_update<float>, BP_UPDATE))) return rc;
    if ((rc = occupancy(kb_finalize<float>, BP_FIN))) return rc;
    // one-CTA-per-simulation passes need no more CTAs than simulations
    grid[BP_SCALAR] = std::min(grid[BP_SCALAR], cfg.max_active);
    grid[BP_FIN] = std::min(grid[BP_FIN], cfg.max_active);
    // size classes with compile-time shapes
    cls[1] = batch_class_ops_32(); cls[2] = batch_class_ops_48(); cls[3] = batch_class_ops_64();
    cls[4] = batch_class_ops_96(); cls[5] = batch_class_ops_128();
    for (int ph = 0; ph < BP_COUNT; ++ph)   // the generic class's tiles
      cl[0].tile[ph] = (ph == BP_X || ph == BP_X_LES) ? LYZB : (ph == BP_INV_Z || ph == BP_INV_Y || ph == BP_FWD_Y ||
                                                                   ph == BP_FWD_Z) ? TXB : 1;
    for (int c = 1; c < BATCH_NCLASS; ++c) {
      if (cls[c].n > cfg.max_n) continue;
      std::string e;
      int form[BP_COUNT] = {0};
      const bool forced = !cfg.autotune && (cfg.class_forms == 1 || cfg.class_forms == 2);
      if (forced)
        for (int ph : {BP_INV_Z, BP_INV_Y, BP_FWD_Y, BP_FWD_Z, BP_X, BP_X_LES})
          form[ph] = (ph == BP_X || ph == BP_X_LES) ? (cfg.class_forms == 1 ? XF_LYZ4 : XF_LYZ2)
                                                    : (cfg.class_forms == 1 ? YZ_TX8 : YZ_TX4);
      if (cfg.autotune && (rc = tune_class(c, form))) return rc;
      if ((rc = cls[c].prepare(cfg.device, cfg.max_active, (cfg.autotune || forced) ? form : nullptr, &cl[c], &e))) {
        terr = e;
        return rc;
      }
    }
    for (int c = 0; c < BATCH_NCLASS; ++c) SV_CK(cudaStreamCreateWithFlags(&cs[c], cudaStreamNonBlocking));
    for (int c = 0; c <= BATCH_NCLASS; ++c) SV_CK(cudaEventCreateWithFlags(&cev[c], cudaEventDisableTiming));

    slots.resize(cfg.max_active);
    SV_CK(cudaMalloc(&d_inst, sizeof(BI) * cfg.max_active));
    SV_CK(cudaMallocHost(&h_inst, sizeof(BI) * cfg.max_active));
    SV_CK(cudaMalloc(&d_tab, sizeof(BatchTables)));
    SV_CK(cudaMallocHost(&h_tab, sizeof(BatchTables)));
    memset(h_tab, 0, sizeof(BatchTables));
    SV_CK(cudaMemcpyAsync(d_tab, h_tab, sizeof(BatchTables), cudaMemcpyHostToDevice, S));
    for (int i = 0; i < 2; ++i) SV_CK(cudaEventCreateWithFlags(&h_ev[i], cudaEventDisableTiming));
    SV_CK(cudaMalloc(&d_health, sizeof(unsigned) * cfg.max_active));
    SV_CK(cudaMallocHost(&h_health, sizeof(unsigned) * cfg.max_active));
    SV_CK(cudaEventCreateWithFlags(&health_ev, cudaEventDisableTiming));
    health_job.assign(cfg.max_active, 0);
    SV_CK(cudaStreamSynchronize(S));
    // the step graph: one launch per pass, each walking its table
    // the step graph: S forks one branch per class; each branch is that class's chain
    SV_CK(cudaStreamBeginCapture(S, cudaStreamCaptureModeThreadLocal));
    SV_CK(cudaEventRecord(cev[BATCH_NCLASS], S));
    for (int c = 0; c < BATCH_NCLASS; ++c) {
      if (c > 0 && cls[c].n > cfg.max_n) continue;
      cudaStream_t b = cs[c];
      SV_CK(cudaStreamWaitEvent(b, cev[BATCH_NCLASS], 0));
      if (c == 0) {
        kb_inv_z<float, TXB><<<grid[BP_INV_Z], block[BP_INV_Z], smem[BP_INV_Z], b>>>(d_inst, d_tab);
        kb_inv_y<float, TXB><<<grid[BP_INV_Y], block[BP_INV_Y], smem[BP_INV_Y], b>>>(d_inst, d_tab);
        kb_x<float, false, LYZB><<<grid[BP_X], block[BP_X], smem[BP_X], b>>>(d_inst, d_tab);
        kb_x<float, true, LYZB><<<grid[BP_X_LES], block[BP_X_LES], smem[BP_X_LES], b>>>(d_inst, d_tab);
        kb_fwd_y<float, TXB><<<grid[BP_FWD_Y], block[BP_FWD_Y], smem[BP_FWD_Y], b>>>(d_inst, d_tab);
        kb_scalar<float><<<grid[BP_SCALAR], block[BP_SCALAR], 0, b>>>(d_inst, d_tab);
        kb_table<float><<<grid[BP_TABLE], block[BP_TABLE], 0, b>>>(d_inst, d_tab);
        kb_fwd_z<float, TXB><<<grid[BP_FWD_Z], block[BP_FWD_Z], smem[BP_FWD_Z], b>>>(d_inst, d_tab);
        kb_stats<float><<<grid[BP_STATS], block[BP_STATS], 0, b>>>(d_inst, d_tab);
        kb_update<float><<<grid[BP_UPDATE], block[BP_UPDATE], 0, b>>>(d_inst, d_tab);
        kb_finalize<float><<<grid[BP_FIN], block[BP_FIN], 0, b>>>(d_inst, d_tab);
      } else {
        cls[c].enqueue(cl[c], b, d_inst, d_tab);
      }
      SV_CK(cudaEventRecord(cev[c], b));
      SV_CK(cudaStreamWaitEvent(S, cev[c], 0));
    }
    cudaError_t e = cudaStreamEndCapture(S, &graph);
    if (e != cudaSuccess) { terr = std::string("graph capture: ") + cudaGetErrorString(e); return FFS_ECUDA; }
    SV_CK(cudaGraphInstantiate(&gexec, graph, 0));
    return 0;
  }

  // Autotuner of one size class: probe simulations of the class's side (enough that a
  // pass's work is close to one 128^3 simulation's), then per tunable pass every kernel
  // form timed on them (work tables cut in that form's tiles, the other passes at their
  // current picks); the fastest form stays. Velocity-only probes time the y/z passes and
  // the x pass, LES probes the LES x pass. The probes are freed afterwards; the choice is
  // kept for the process.
  int tune_class(int c, int form[BP_COUNT]) {
    const ClassOps& ops = cls[c];
    const int n = ops.n;
    std::string e;
    ClassLaunch L{};
    int rc = ops.prepare(cfg.device, cfg.max_active, nullptr, &L, &e);
    if (rc) { terr = e; return rc; }
    for (int ph = 0; ph < BP_COUNT; ++ph) form[ph] = L.form[ph];
    const std::string key = std::to_string(cfg.device) + ":" + std::to_string(n) + ":" + std::to_string(cfg.max_active);
    {
      std::lock_guard<std::mutex> g(class_tune_mu());
      auto it = class_tune_cache().find(key);
      if (it != class_tune_cache().end()) {
        for (int ph = 0; ph < BP_COUNT; ++ph) form[ph] = it->second.form[ph];
        tune_report += it->second.report + " (cached); ";
        return 0;
      }
    }
    const int want = std::max(1, (128 / n) * (128 / n) * (128 / n));
    const size_t N = (size_t)n * n * n;
    std::vector<double> u(3 * N);
    for (int z = 0; z < n; ++z)   // a smooth divergence-free field: (sin y, sin z, sin x)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          const size_t i = ((size_t)z * n + y) * n + x;
          u[i] = sin(2 * M_PI * y / n); u[N + i] = sin(2 * M_PI * z / n); u[2 * N + i] = sin(2 * M_PI * x / n);
        }
    std::vector<std::unique_ptr<EngineBase>> probes;
    std::vector<BatchGeom> geo[2];
    std::vector<BI> hb;
    for (int les = 0; les < 2; ++les) {
      ffs_params p;
      ffs_params_default(&p);
      p.nx = p.ny = p.nz = n; p.precision = FFS_FP32; p.integrator = FFS_AB3; p.variable_dt = 1; p.cfl = 0.2;
      p.nu = 1e-3; p.dt_stat = p.dt_spec = 1 << 30; p.les = les; p.device = cfg.device;
      const int64_t pb = std::max<int64_t>(1, estimate_bytes_f32(p));
      const int64_t fit = std::max<int64_t>(1, cfg.memory_budget / 4 / pb);
      const int k = (int)std::min<int64_t>({(int64_t)want, (int64_t)cfg.max_active, (int64_t)64, fit});
      for (int i = 0; i < k; ++i) {
        std::unique_ptr<EngineBase> eng(make_engine_f32());
        BatchGeom g{};
        BI b{};
        if ((rc = eng->create(p, e)) || (rc = eng->set_fields(u.data(), u.data() + N, u.data() + 2 * N, nullptr, 0, e)) ||
            (rc = eng->initialize(e)) || (rc = eng->batch_export(&b, sizeof(BI), &g, e))) {
          terr = "size class tuning: " + e;
          return rc;
        }
        geo[les].push_back(g);
        hb.push_back(b);
        probes.push_back(std::move(eng));
      }
    }
    const int base[2] = {0, (int)geo[0].size()};
    BI* d_b = nullptr;
    BatchTables* d_t = nullptr;
    WorkItem* d_it = nullptr;
    size_t cap = 0;
    cudaEvent_t a = nullptr, b = nullptr;
    auto cleanup = [&] {
      if (d_b) cudaFree(d_b);
      if (d_t) cudaFree(d_t);
      if (d_it) cudaFree(d_it);
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
    };
    auto ck = [&](cudaError_t r, const char* what) {
      if (r != cudaSuccess && !rc) { terr = std::string("size class tuning: ") + what + ": " + cudaGetErrorString(r); rc = FFS_ECUDA; }
      return r == cudaSuccess;
    };
    std::string rep = "n=" + std::to_string(n) + " (" + std::to_string(geo[0].size()) + "+" +
                      std::to_string(geo[1].size()) + " probes):";
    if (ck(cudaMalloc(&d_b, sizeof(BI) * hb.size()), "malloc") && ck(cudaMalloc(&d_t, sizeof(BatchTables)), "malloc") &&
        ck(cudaMemcpy(d_b, hb.data(), sizeof(BI) * hb.size(), cudaMemcpyHostToDevice), "upload") &&
        ck(cudaEventCreate(&a), "event") && ck(cudaEventCreate(&b), "event")) {
      const char* pn[BP_COUNT] = {"inv_z", "inv_y", "x", "x_les", "fwd_y", "", "", "fwd_z", "", "", ""};
      const char* fn_yz[3] = {"pair", "tx8", "tx4"};
      const char* fn_x[3] = {"fused", "lyz4", "lyz2"};
      for (int ph : {BP_INV_Z, BP_INV_Y, BP_X, BP_FWD_Y, BP_FWD_Z, BP_X_LES}) {
        const unsigned m = ops.forms(ph);
        if (rc || __builtin_popcount(m) < 2) continue;
        const int set = ph == BP_X_LES ? 1 : 0;
        float best = 1e30f;
        int bf = form[ph];
        for (int f = 0; f < 3 && !rc; ++f) {
          if (!((m >> f) & 1u)) continue;
          int fc[BP_COUNT];
          for (int q = 0; q < BP_COUNT; ++q) fc[q] = form[q];
          fc[ph] = f;
          ClassLaunch Lc{};
          if (ops.prepare(cfg.device, cfg.max_active, fc, &Lc, &e)) continue;   // form does not fit
          std::vector<WorkItem> items;
          for (size_t i = 0; i < geo[set].size(); ++i) append_items(ph, Lc.tile[ph], geo[set][i], base[set] + (int)i, items);
          if (items.size() > cap) {
            if (d_it) cudaFree(d_it);
            d_it = nullptr;
            cap = items.size();
            if (!ck(cudaMalloc(&d_it, sizeof(WorkItem) * cap), "malloc")) break;
          }
          BatchTables t{};
          t.tab[c][ph] = d_it;
          t.n[c][ph] = (int)items.size();
          if (!ck(cudaMemcpy(d_it, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice), "upload") ||
              !ck(cudaMemcpy(d_t, &t, sizeof(t), cudaMemcpyHostToDevice), "upload"))
            break;
          const int reps = n >= 96 ? 10 : 20;
          ops.launch(Lc, ph, S, d_b, d_t);
          ck(cudaEventRecord(a, S), "event");
          for (int r = 0; r < reps; ++r) ops.launch(Lc, ph, S, d_b, d_t);
          ck(cudaEventRecord(b, S), "event");
          ck(cudaEventSynchronize(b), "synchronize");
          ck(cudaGetLastError(), "launch");
          float ms = 0.f;
          ck(cudaEventElapsedTime(&ms, a, b), "timing");
          ms /= reps;
          char line[96];
          snprintf(line, sizeof(line), " %s[%s]=%.4fms", pn[ph], (ph == BP_X || ph == BP_X_LES) ? fn_x[f] : fn_yz[f], ms);
          rep += line;
          if (ms < best) { best = ms; bf = f; }
        }
        form[ph] = bf;
      }
    }
    cleanup();
    probes.clear();
    if (rc) return rc;
    rep += " ->";
    for (int ph : {BP_INV_Z, BP_INV_Y, BP_X, BP_X_LES, BP_FWD_Y, BP_FWD_Z}) rep += " " + std::to_string(form[ph]);
    tune_report += rep + "; ";
    std::lock_guard<std::mutex> g(class_tune_mu());
    ClassTune ct;
    for (int ph = 0; ph < BP_COUNT; ++ph) ct.form[ph] = form[ph];
    ct.report = rep;
    class_tune_cache()[key] = ct;
    return 0;
  }

  void release_gpu() {
    if (S) cudaStreamSynchronize(S);
    slots.clear();   // engines free their own buffers and streams
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr; graph = nullptr;
    if (d_items) cudaFree(d_items);
    for (int i = 0; i < 2; ++i) {
      if (h_items[i]) cudaFreeHost(h_items[i]);
      if (h_ev[i]) cudaEventDestroy(h_ev[i]);
      h_items[i] = nullptr; h_ev[i] = nullptr;
    }
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    ev_pool.clear();
    if (d_inst) cudaFree(d_inst);
    if (h_inst) cudaFreeHost(h_inst);
    if (d_health) cudaFree(d_health);
    if (h_health) cudaFreeHost(h_health);
    if (health_ev) cudaEventDestroy(health_ev);
    d_health = nullptr; h_health = nullptr; health_ev = nullptr;
    if (d_tab) cudaFree(d_tab);
    if (h_tab) cudaFreeHost(h_tab);
    d_items = nullptr; d_inst = nullptr; h_inst = nullptr; d_tab = nullptr; h_tab = nullptr;
    for (int c = 0; c < BATCH_NCLASS; ++c) {
      if (cs[c]) cudaStreamDestroy(cs[c]);
      cs[c] = nullptr;
    }
    for (int c = 0; c <= BATCH_NCLASS; ++c) {
      if (cev[c]) cudaEventDestroy(cev[c]);
      cev[c] = nullptr;
    }
    if (S) cudaStreamDestroy(S);
    S = nullptr;
  }

  void shutdown() {
    {
      std::lock_guard<std::mutex> g(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (th.joinable()) th.join();
    release_gpu();
  }

  // ------------------------------------------------------------------ API side
  int fail_api(int code, const std::string& m) {
    std::lock_guard<std::mutex> g(mu);
    err = m;
    return code;
  }
  std::string last_error() {
    std::lock_guard<std::mutex> g(mu);
    return err;
  }

  int submit(const ffs_request& r, uint64_t* id) {
    const ffs_params& p = r.params;
    if (p.precision != FFS_FP32) return fail_api(FFS_EUNSUPPORTED, "the server runs FP32 simulations only");
    if (p.plane_forcing) return fail_api(FFS_EUNSUPPORTED, "the server does not batch kz = 0 plane forcing");
    if (p.density || p.passive_scalar)
      return fail_api(FFS_EUNSUPPORTED, "the server does not batch density-stratified or passive-scalar runs");
    if (p.les && (p.les_model != FFS_LES_SMAGORINSKY || p.sandp_cb != 0.0))
      return fail_api(FFS_EUNSUPPORTED, "the server batches the Smagorinsky LES model only");
    if (p.spec_fil != 0.0) return fail_api(FFS_EUNSUPPORTED, "the server does not batch filtered statistics (specFil)");
    int tpl, np;
    for (int n : {p.nx, p.ny, p.nz}) {
      plan_shape(n, tpl, np);
      if (!tpl || n > cfg.max_n)
        return fail_api(FFS_EUNSUPPORTED, "grid side " + std::to_string(n) +
                                              " not served (sides 8..128 of the engine's list, <= max_n)");
    }
    if (((long long)p.ny * p.nz) % LYZB) return fail_api(FFS_EUNSUPPORTED, "ny*nz must be a multiple of 4");
    if (r.nt < 0) return fail_api(FFS_EINVAL, "nt must be >= 0");
    if (!r.u1 || !r.u2 || !r.u3) return fail_api(FFS_EINVAL, "velocity pointers must not be NULL");
    auto j = std::make_shared<Job>();
    j->p = p;
    j->p.device = cfg.device;
    j->p.kernel_variant = 0;   // engines carry the fused x passes' twiddles (64^3, 128^3)
    // records of one run stay on the device until it finishes
    j->p.stats_capacity = (int32_t)std::max<int64_t>(64, r.nt / std::max(1, p.dt_stat) + 4);
    j->p.spec_capacity = (int32_t)std::max<int64_t>(4, r.nt / std::max(1, p.dt_spec) + 4);
    j->nt = r.nt;
    j->keep_fields = r.keep_fields;
    const size_t N = (size_t)p.nx * p.ny * p.nz;
    j->u.resize(3 * N);
    memcpy(j->u.data(), r.u1, sizeof(double) * N);
    memcpy(j->u.data() + N, r.u2, sizeof(double) * N);
    memcpy(j->u.data() + 2 * N, r.u3, sizeof(double) * N);
    {
      std::lock_guard<std::mutex> g(mu);
      if (!fatal.empty()) { err = "server stopped: " + fatal; return FFS_ESTATE; }
      j->id = next_id++;
      j->t_submit = now_s(t0);
      queue.push_back(j);
      jobs[j->id] = j;
      info.queued = (int32_t)queue.size();
      *id = j->id;
    }
    cv_work.notify_all();
    return 0;
  }

  void fill(const Job& j, ffs_result* o) {
    // a failed request's message becomes the server's last error (mu is held)
    if (j.status < 0) err = "request " + std::to_string(j.id) + ": " + j.err;
    o->status = j.status;
    o->iteration = j.iteration;
    o->time = j.time;
    o->dt = j.dt;
    o->stats_rows = j.ncols ? (int64_t)j.stats.size() / j.ncols : 0;
    o->record_ncols = j.ncols;
    o->submit_s = j.t_submit;
    o->admit_s = j.t_admit;
    o->done_s = j.t_done;
  }

  int poll(uint64_t id, ffs_result* o) {
    std::lock_guard<std::mutex> g(mu);
    auto it = jobs.find(id);
    if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
    fill(*it->second, o);
    return 0;
  }

  int wait(uint64_t id, double timeout_s, ffs_result* o) {
    std::unique_lock<std::mutex> g(mu);
    auto it = jobs.find(id);
    if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
    std::shared_ptr<Job> j = it->second;
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (j->status == FFS_QUEUED || j->status == FFS_RUNNING) {
      if (!fatal.empty()) { err = "server stopped: " + fatal; return FFS_ESTATE; }
      if (cv_done.wait_until(g, until) == std::cv_status::timeout &&
          (j->status == FFS_QUEUED || j->status == FFS_RUNNING)) {
        fill(*j, o);
        return FFS_ETIMEDOUT;
      }
    }
    fill(*j, o);
    return 0;
  }

  int64_t fetch_stats(uint64_t id, double* out, int64_t max_rows) {
    std::lock_guard<std::mutex> g(mu);
    auto it = jobs.find(id);
    if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
    const Job& j = *it->second;
    if (j.status == FFS_QUEUED || j.status == FFS_RUNNING) { err = "request not finished"; return FFS_ESTATE; }
    const int64_t have = j.ncols ? (int64_t)j.stats.size() / j.ncols : 0;
    if (!out) return have;
    const int64_t n = std::min(have, max_rows);
    memcpy(out, j.stats.data(), sizeof(double) * n * j.ncols);
    return n;
  }

  int fetch_fields(uint64_t id, double* u1, double* u2, double* u3) {
    std::lock_guard<std::mutex> g(mu);
    auto it = jobs.find(id);
    if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
    const Job& j = *it->second;
    if (j.status != FFS_OK) { err = "request not finished"; return FFS_ESTATE; }
    if (j.fields.empty()) { err = "request was submitted without keep_fields"; return FFS_ESTATE; }
    const size_t N = j.fields.size() / 3;
    double* d[3] = {u1, u2, u3};
    for (int c = 0; c < 3; ++c)
      if (d[c]) memcpy(d[c], j.fields.data() + c * N, sizeof(double) * N);
    return 0;
  }

  // cancel a queued or running request: a queued one leaves the queue now, a pending or
  // running one when the serving thread next looks (before its next replay)
  int cancel(uint64_t id) {
    std::shared_ptr<Job> j;
    {
      std::lock_guard<std::mutex> g(mu);
      auto it = jobs.find(id);
      if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
      j = it->second;
      if (j->status != FFS_QUEUED && j->status != FFS_RUNNING) { err = "request already finished"; return FFS_ESTATE; }
      j->cancel = true;
      auto q = std::find(queue.begin(), queue.end(), j);
      if (q == queue.end()) {
        cv_work.notify_all();
        return 0;
      }
      queue.erase(q);
      info.queued = (int32_t)queue.size();
    }
    finish_job(j, FFS_ECANCELED, "cancelled while queued");
    return 0;
  }

  int release(uint64_t id) {
    std::lock_guard<std::mutex> g(mu);
    auto it = jobs.find(id);
    if (it == jobs.end()) { err = "unknown request id"; return FFS_EINVAL; }
    if (it->second->status == FFS_QUEUED || it->second->status == FFS_RUNNING) {
      err = "request still pending";
      return FFS_ESTATE;
    }
    jobs.erase(it);
    return 0;
  }

  int pause(int on) {
    {
      std::lock_guard<std::mutex> g(mu);
      paused = on != 0;
    }
    cv_work.notify_all();
    return 0;
  }

  int stats(ffs_server_info* o) {
    std::lock_guard<std::mutex> g(mu);
    *o = info;
    return 0;
  }

  // ------------------------------------------------------------------ serving thread
  void finish_job(const std::shared_ptr<Job>& j, int status, const std::string& msg) {
    std::lock_guard<std::mutex> g(mu);
    j->status = status;
    j->err = msg;
    j->t_done = now_s(t0);
    j->u.clear();
    j->u.shrink_to_fit();
    cv_done.notify_all();
  }

  static bool same_buffers(const ffs_params& a, const ffs_params& b) {
    return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.lx == b.lx && a.ly == b.ly && a.lz == b.lz &&
           a.cutoff == b.cutoff && a.integrator == b.integrator && (a.les != 0) == (b.les != 0) &&
           (a.forcing != 0) == (b.forcing != 0) && (a.hyperviscosity != 0) == (b.hyperviscosity != 0) &&
           a.stats_capacity <= b.stats_capacity && a.spec_capacity <= b.spec_capacity;
  }

  // admit one job into slot k (k idle or empty); returns false if it must wait
  bool admit(const std::shared_ptr<Job>& j, std::vector<int>& dirty) {
    int k = -1;
    // 1. an idle pooled engine with the same buffers
    for (int i = 0; i < (int)slots.size(); ++i)
      if (slots[i].eng && !slots[i].job && !slots[i].retiring && same_buffers(j->p, slots[i].p)) { k = i; break; }
    std::string e;
    if (k >= 0) {
      if (slots[k].eng->repurpose(j->p, e)) {
        finish_job(j, FFS_EINVAL, e);
        return true;
      }
    } else {
      const int64_t need = estimate_bytes_f32(j->p);
      if (need < 0) { finish_job(j, FFS_EUNSUPPORTED, "unsupported grid"); return true; }
      if (need > cfg.memory_budget) { finish_job(j, FFS_ENOMEM, "request exceeds the server's memory budget"); return true; }
      // free idle pooled engines until it fits
      while (bytes_in_use + need > cfg.memory_budget) {
        int victim = -1;
        for (int i = 0; i < (int)slots.size(); ++i)
          if (slots[i].eng && !slots[i].job && !slots[i].retiring) { victim = i; break; }
        if (victim < 0) return false;
        bytes_in_use -= slots[victim].bytes;
        slots[victim].eng.reset();
        slots[victim].bytes = 0;
      }
      for (int i = 0; i < (int)slots.size(); ++i)
        if (!slots[i].eng && !slots[i].retiring) { k = i; break; }
      if (k < 0) {   // every slot holds an engine: drop an idle one of another shape
        for (int i = 0; i < (int)slots.size(); ++i)
          if (slots[i].eng && !slots[i].job && !slots[i].retiring) { k = i; break; }
        if (k < 0) return false;
        bytes_in_use -= slots[k].bytes;
        slots[k].eng.reset();
        slots[k].bytes = 0;
      }
      std::unique_ptr<EngineBase> eng(make_engine_f32());
      const int rc = eng->create(j->p, e);
      if (rc) {
        finish_job(j, rc, e);
        return true;
      }
      slots[k].eng = std::move(eng);
      slots[k].p = j->p;
      slots[k].bytes = slots[k].eng->device_bytes();
      bytes_in_use += slots[k].bytes;
    }
    Slot& s = slots[k];
    const size_t N = (size_t)j->p.nx * j->p.ny * j->p.nz;
    int rc = s.eng->set_fields(j->u.data(), j->u.data() + N, j->u.data() + 2 * N, nullptr, 0, e);
    if (!rc) rc = s.eng->initialize(e);
    BatchGeom g{};
    // the pinned mirror of slot k may still feed an upload in flight
    if (!rc && (cudaEventSynchronize(h_ev[0]) != cudaSuccess || cudaEventSynchronize(h_ev[1]) != cudaSuccess)) {
      rc = FFS_ECUDA;
      e = "event synchronize failed";
    }
    if (!rc) rc = s.eng->batch_export(&h_inst[k], sizeof(BI), &g, e);
    if (!rc && (g.txy != TXB || g.txz != TXB || g.lyz != LYZB || g.density)) {
      rc = FFS_EUNSUPPORTED;
      e = "grid needs launch tiles the batch does not use";
    }
    if (rc) {
      finish_job(j, rc, e);
      return true;
    }
    s.g = g;
    s.job = j;
    s.done = 0;
    s.it0 = s.eng->iteration;
    {
      std::lock_guard<std::mutex> gl(mu);
      j->status = FFS_RUNNING;
      j->t_admit = now_s(t0);
      j->u.clear();
      j->u.shrink_to_fit();
    }
    if (j->nt == 0) {   // nothing to step: the results are the initialized state
      retire(k, nullptr);
      return true;
    }
    dirty.push_back(k);
    return true;
  }

  // the classes whose x pass is register-fused for this model (they need the engine's
  // register-pass twiddles): 64^3 and 128^3, velocity-only and LES
  static bool fused_x(const BatchGeom& g) { return g.nx == 64 || g.nx == 128; }
  // size class of a simulation: its cubic side when a class exists for it, else the
  // generic class
  int class_of(const BatchGeom& g) const {
    if (g.nx != g.ny || g.nx != g.nz) return 0;
    for (int c = 1; c < BATCH_NCLASS; ++c)
      if (cls[c].n == g.nx && g.nx <= cfg.max_n) return (fused_x(g) && g.xfused != g.nx) ? 0 : c;
    return 0;
  }

  // work tables of the simulations in the batch, per class
  std::vector<WorkItem> items[BATCH_NCLASS][BP_COUNT];
  int rebuild_tables(const std::vector<int>& dirty) {
    for (auto& c : items)
      for (auto& v : c) v.clear();
    for (int k = 0; k < (int)slots.size(); ++k) {
      const Slot& s = slots[k];
      if (!s.job || s.retiring) continue;
      const BatchGeom& g = s.g;
      const int c = class_of(g);
      auto& it = items[c];
      const int xph = g.les ? BP_X_LES : BP_X;
      for (int ph : {(int)BP_INV_Z, (int)BP_INV_Y, xph, (int)BP_FWD_Y, (int)BP_FWD_Z}) append_items(ph, cl[c].tile[ph], g, k, it[ph]);
      it[BP_SCALAR].push_back({k, 0, 0, 0});
      for (int b = 0; b < g.table_blocks; ++b) it[BP_TABLE].push_back({k, b, g.table_blocks, 0});
      for (int b = 0; b < g.nparts; ++b) it[BP_STATS].push_back({k, b, g.nparts, 0});
      for (int b = 0; b < g.upd_blocks; ++b) it[BP_UPDATE].push_back({k, b, g.upd_blocks, 0});
      it[BP_FIN].push_back({k, 0, 0, 0});
    }
    size_t total = 0;
    for (auto& c : items)
      for (auto& v : c) total += v.size();
    total = std::max<size_t>(total, 1);
    // device table storage (grows; the descriptor carries the pointers)
    if (total > d_cap) {
      SV_CK(cudaStreamSynchronize(S));
      if (d_items) SV_CK(cudaFree(d_items));
      d_cap = std::max(total, 2 * d_cap);
      SV_CK(cudaMalloc(&d_items, sizeof(WorkItem) * d_cap));
    }
    // pinned staging: wait until its previous upload finished
    int b = h_cur;
    h_cur ^= 1;
    SV_CK(cudaEventSynchronize(h_ev[b]));
    if (total > h_cap[b]) {
      if (h_items[b]) SV_CK(cudaFreeHost(h_items[b]));
      h_cap[b] = std::max(total, 2 * h_cap[b]);
      SV_CK(cudaMallocHost(&h_items[b], sizeof(WorkItem) * h_cap[b]));
    }
    size_t off = 0;
    BatchTables t{};
    for (int c = 0; c < BATCH_NCLASS; ++c)
      for (int ph = 0; ph < BP_COUNT; ++ph) {
        const auto& v = items[c][ph];
        memcpy(h_items[b] + off, v.data(), sizeof(WorkItem) * v.size());
        t.tab[c][ph] = d_items + off;
        t.n[c][ph] = (int)v.size();
        off += v.size();
      }
    SV_CK(cudaEventSynchronize(h_ev[b ^ 1]));   // h_tab / h_inst are shared by both buffers
    *h_tab = t;
    for (int k : dirty) SV_CK(cudaMemcpyAsync(d_inst + k, h_inst + k, sizeof(BI), cudaMemcpyHostToDevice, S));
    SV_CK(cudaMemcpyAsync(d_items, h_items[b], sizeof(WorkItem) * std::max<size_t>(off, 1), cudaMemcpyHostToDevice, S));
    SV_CK(cudaMemcpyAsync(d_tab, h_tab, sizeof(BatchTables), cudaMemcpyHostToDevice, S));
    SV_CK(cudaEventRecord(h_ev[b], S));
    return 0;
  }

  cudaEvent_t get_event() {
    if (!ev_pool.empty()) {
      cudaEvent_t e = ev_pool.back();
      ev_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
  }

  // read a finished simulation's results on its own stream, after its last step
  void retire(int k, cudaEvent_t ev) {
    Slot& s = slots[k];
    std::shared_ptr<Job> j = s.job;
    std::string e;
    int rc = ev ? s.eng->stream_wait(ev, e) : 0;
    const int64_t steps = s.early ? s.done : j->nt;   // steps the simulation took in the batch
    if (!rc && steps > 0) rc = s.eng->sync_host_state(s.it0, s.it0 + steps - 1, e);
    if (s.early == FFS_ENAN && rc == 0) {   // the flag was seen; the drain did not (cannot happen)
      rc = FFS_ENAN;
      e = "non-finite value in the spectral state (simulation diverged)";
    }
    if (s.early == FFS_ECANCELED) {
      rc = FFS_ECANCELED;
      e = "cancelled after " + std::to_string(s.done) + " of " + std::to_string(j->nt) + " steps";
    } else if (s.early == FFS_ENAN) {
      e += "; retired after " + std::to_string(s.done) + " of " + std::to_string(j->nt) + " steps";
    }
    std::vector<double> fields;
    if (!rc && j->keep_fields) {
      const size_t N = (size_t)j->p.nx * j->p.ny * j->p.nz;
      fields.resize(3 * N);
      rc = s.eng->get_fields(fields.data(), fields.data() + N, fields.data() + 2 * N, nullptr, 0, e);
    }
    {
      std::lock_guard<std::mutex> g(mu);
      j->ncols = s.eng->ncols_rec;
      j->stats.swap(s.eng->rec_host);
      j->fields.swap(fields);
      j->iteration = s.eng->iteration;
      j->time = s.eng->time;
      j->dt = s.eng->dt;
    }
    finish_job(j, rc, e);
    s.job.reset();
    s.retiring = false;
    s.early = 0;
  }

  // Health snapshot and cancellations, before the next replay. A simulation found
  // diverged (its update saw a non-finite value) or cancelled leaves the tables now; its
  // results are read after the replays already queued for it, like a normal finisher's.
  void check_early(int& active, bool& changed, std::vector<std::pair<int, cudaEvent_t>>& retiring) {
    std::vector<int> out;
    int64_t bs;
    {
      std::lock_guard<std::mutex> g(mu);
      bs = info.batch_steps;
    }
    // a snapshot one interval old is waited for: the host then never runs more than two
    // intervals of replays ahead of the GPU, which bounds how long a diverged simulation
    // keeps its slot
    if (health_pending && (bs - health_at >= kHealthEvery ? cudaEventSynchronize(health_ev)
                                                           : cudaEventQuery(health_ev)) == cudaSuccess) {
      health_pending = false;
      for (int k = 0; k < (int)slots.size(); ++k) {
        Slot& s = slots[k];
        if (s.job && !s.retiring && health_job[k] == s.job->id && (h_health[k] & 1u)) {
          s.early = FFS_ENAN;
          out.push_back(k);
        }
      }
    }
    {
      std::lock_guard<std::mutex> g(mu);
      for (int k = 0; k < (int)slots.size(); ++k) {
        Slot& s = slots[k];
        if (s.job && !s.retiring && !s.early && s.job->cancel) {
          s.early = FFS_ECANCELED;
          out.push_back(k);
        }
      }
    }
    if (out.empty()) return;
    cudaEvent_t ev = get_event();
    cudaEventRecord(ev, S);   // after every replay enqueued so far
    for (int k : out) {
      slots[k].retiring = true;
      --active;
      changed = true;
      retiring.push_back({k, ev});
    }
  }

  // enqueue a health snapshot behind the replays enqueued so far
  void snapshot_health() {
    if (health_pending) return;
    cudaMemsetAsync(d_health, 0, sizeof(unsigned) * slots.size(), S);
    k_batch_health<<<1, 256, 0, S>>>(d_inst, d_tab, d_health);
    cudaMemcpyAsync(h_health, d_health, sizeof(unsigned) * slots.size(), cudaMemcpyDeviceToHost, S);
    for (int k = 0; k < (int)slots.size(); ++k)
      health_job[k] = (slots[k].job && !slots[k].retiring) ? slots[k].job->id : 0;
    cudaEventRecord(health_ev, S);
    health_pending = true;
    std::lock_guard<std::mutex> g(mu);
    health_at = info.batch_steps;
  }

  void loop() {
    cudaSetDevice(cfg.device);
    std::deque<std::shared_ptr<Job>> pending;
    std::vector<std::pair<int, cudaEvent_t>> retiring;   // finished at the last replay
    int active = 0;
    bool changed = false;
    std::vector<int> dirty;
    auto fail = [&](const std::string& m) {
      std::lock_guard<std::mutex> g(mu);
      fatal = m;
      for (auto& kv : jobs)
        if (kv.second->status == FFS_QUEUED || kv.second->status == FFS_RUNNING) {
          kv.second->status = FFS_ECUDA;
          kv.second->err = m;
        }
      cv_done.notify_all();
    };
    while (true) {
      {
        std::unique_lock<std::mutex> g(mu);
        if (stop) break;
        if (active == 0 && retiring.empty() && (queue.empty() || paused) && pending.empty())
          cv_work.wait_for(g, std::chrono::milliseconds(50));
        if (stop) break;
        if (!paused)
          while (!queue.empty()) { pending.push_back(queue.front()); queue.pop_front(); }
      }
      // admission (a request cancelled after it left the queue is dropped here)
      {
        std::vector<std::shared_ptr<Job>> dropped;
        {
          std::lock_guard<std::mutex> g(mu);
          for (auto it = pending.begin(); it != pending.end();) {
            if ((*it)->cancel) { dropped.push_back(*it); it = pending.erase(it); }
            else ++it;
          }
        }
        for (auto& j : dropped) finish_job(j, FFS_ECANCELED, "cancelled before admission");
      }
      while (!pending.empty() && active < cfg.max_active) {
        if (!admit(pending.front(), dirty)) break;
        const bool running = pending.front()->status == FFS_RUNNING;
        pending.pop_front();
        if (running) { ++active; changed = true; }
      }
      {
        std::lock_guard<std::mutex> g(mu);
        info.queued = (int32_t)(pending.size() + queue.size());
        info.active = active;
        info.peak_active = std::max(info.peak_active, active);
        info.bytes_in_use = bytes_in_use;
        info.peak_bytes = std::max(info.peak_bytes, bytes_in_use);
      }
      if (active > 0) check_early(active, changed, retiring);
      if (changed) {
        if (rebuild_tables(dirty)) { fail(err); break; }
        dirty.clear();
        changed = false;
      }
      if (active > 0) {
        if (cudaGraphLaunch(gexec, S) != cudaSuccess) { fail("graph launch failed"); break; }
        cudaEvent_t ev = get_event();
        cudaEventRecord(ev, S);
        // simulations finished by this replay leave the tables before the next one
        std::vector<std::pair<int, cudaEvent_t>> now;
        int sims = 0;
        for (int k = 0; k < (int)slots.size(); ++k) {
          Slot& s = slots[k];
          if (!s.job || s.retiring) continue;
          ++s.done;
          ++sims;
          if (s.done >= s.job->nt) {
            s.retiring = true;
            --active;
            changed = true;
            now.push_back({k, ev});
          }
        }
        int64_t bs;
        {
          std::lock_guard<std::mutex> g(mu);
          info.batch_steps += 1;
          info.sim_steps += sims;
          bs = info.batch_steps;
        }
        if (bs % kHealthEvery == 0) snapshot_health();
        if (now.empty()) ev_pool.push_back(ev);
        // results of the previous replay's finishers, while this replay runs
        for (auto& r : retiring) retire(r.first, r.second);
        std::vector<cudaEvent_t> used;
        for (auto& r : retiring) used.push_back(r.second);
        retiring.swap(now);
        release_events(used, retiring);
      } else if (!retiring.empty()) {
        for (auto& r : retiring) retire(r.first, r.second);
        std::vector<cudaEvent_t> used;
        for (auto& r : retiring) used.push_back(r.second);
        retiring.clear();
        release_events(used, retiring);
      }
    }
    cudaStreamSynchronize(S);
  }

  void release_events(std::vector<cudaEvent_t>& used, const std::vector<std::pair<int, cudaEvent_t>>& keep) {
    std::sort(used.begin(), used.end());
    used.erase(std::unique(used.begin(), used.end()), used.end());
    for (cudaEvent_t e : used) {
      bool held = false;
      for (auto& r : keep) held |= r.second == e;
      if (!held) ev_pool.push_back(e);
    }
  }
};

}  // namespace ffsgpu

struct ffs_server {
  ffsgpu::Server s;
};

namespace {
thread_local std::string g_server_err;
}

extern "C" {

int ffs_server_default(ffs_server_cfg* c) {
  if (!c) return FFS_EINVAL;
  memset(c, 0, sizeof(*c));
  c->device = 0;
  c->memory_budget = 120ll << 30;
  c->max_active = 256;
  c->max_n = 128;
  return FFS_OK;
}

int ffs_server_create(const ffs_server_cfg* c, ffs_server** out) {
  if (!c || !out) return FFS_EINVAL;
  *out = nullptr;
  ffs_server* s = nullptr;
  try {
    s = new ffs_server();
    const int rc = s->s.start(*c);
    if (rc) {
      g_server_err = s->s.err;
      delete s;
      return rc;
    }
  } catch (const std::exception& e) {
    g_server_err = std::string("internal error: ") + e.what();
    delete s;
    return FFS_ENOMEM;
  }
  *out = s;
  return FFS_OK;
}

#define FFS_SERVER_GUARD(expr)                          \
  if (!s) return FFS_EINVAL;                            \
  try {                                                 \
    return (expr);                                      \
  } catch (const std::exception& e) {                   \
    s->s.err = std::string("internal error: ") + e.what(); \
    return FFS_ENOMEM;                                  \
  }

int ffs_submit(ffs_server* s, const ffs_request* r, uint64_t* id) {
  if (!r || !id) return FFS_EINVAL;
  FFS_SERVER_GUARD(s->s.submit(*r, id))
}
int ffs_poll(ffs_server* s, uint64_t id, ffs_result* o) {
  if (!o) return FFS_EINVAL;
  FFS_SERVER_GUARD(s->s.poll(id, o))
}
int ffs_wait(ffs_server* s, uint64_t id, double timeout_s, ffs_result* o) {
  if (!o) return FFS_EINVAL;
  FFS_SERVER_GUARD(s->s.wait(id, timeout_s, o))
}
int64_t ffs_fetch_stats(ffs_server* s, uint64_t id, double* out, int64_t max_rows) {
  FFS_SERVER_GUARD(s->s.fetch_stats(id, out, max_rows))
}
int ffs_fetch_fields(ffs_server* s, uint64_t id, double* u1, double* u2, double* u3) {
  FFS_SERVER_GUARD(s->s.fetch_fields(id, u1, u2, u3))
}
int ffs_release(ffs_server* s, uint64_t id) { FFS_SERVER_GUARD(s->s.release(id)) }
int ffs_cancel(ffs_server* s, uint64_t id) { FFS_SERVER_GUARD(s->s.cancel(id)) }
int ffs_server_pause(ffs_server* s, int32_t paused) { FFS_SERVER_GUARD(s->s.pause(paused)) }
int ffs_server_stats(ffs_server* s, ffs_server_info* o) {
  if (!o) return FFS_EINVAL;
  FFS_SERVER_GUARD(s->s.stats(o))
}
int64_t ffs_server_tuning(ffs_server* s, char* buf, int64_t len) {
  if (!s) return FFS_EINVAL;
  const std::string& r = s->s.tune_report;
  if (buf && len > 0) {
    const size_t m = std::min<size_t>((size_t)len - 1, r.size());
    memcpy(buf, r.data(), m);
    buf[m] = 0;
  }
  return (int64_t)r.size();
}
const char* ffs_server_last_error(ffs_server* s) {
  if (s) g_server_err = s->s.last_error();
  return g_server_err.c_str();
}
void ffs_server_destroy(ffs_server* s) { delete s; }

}  // extern "C"
