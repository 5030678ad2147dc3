// Batched step kernels: many independent simulations (uneven grids) advance together,
// one launch per pass. Each launch is a persistent grid that walks a work table of
// (simulation, block coordinates) entries and runs the same per-block code as the
// single-simulation kernels on that simulation's parameters and buffers. The tables and
// the per-simulation parameter blocks live in device memory at fixed addresses, so one
// captured CUDA graph serves every membership of the batch: admitting or retiring a
// simulation rewrites the tables, not the graph.
//
// Simulations are grouped in size classes. Class 0 takes any grid with runtime FFT
// plans and launch shapes sized for the largest accepted grid; classes 1.. take one
// cubic side each (ffs_batch_class.cuh), with compile-time plans, CTAs of exactly the
// size the plan needs and, for 128^3 velocity-only runs, the register-fused x pass.
// Each class is its own chain of launches; the chains are parallel branches of the
// graph, so classes overlap on the GPU.
#pragma once
#include <string>

#include "ffs_kernels.cuh"

namespace ffsgpu {

struct WorkItem { int inst, x, y, z; };

// The passes of one batched step, in launch order.
enum BatchPhase : int {
  BP_INV_Z = 0, BP_INV_Y, BP_X, BP_X_LES, BP_FWD_Y, BP_SCALAR, BP_TABLE, BP_FWD_Z, BP_STATS, BP_UPDATE, BP_FIN,
  BP_COUNT
};

// size classes: 0 generic, then one per cubic side
constexpr int BATCH_NCLASS = 6;
constexpr int kBatchClassN[BATCH_NCLASS] = {0, 32, 48, 64, 96, 128};

struct BatchTables {
  WorkItem* tab[BATCH_NCLASS][BP_COUNT];
  int n[BATCH_NCLASS][BP_COUNT];
};

template <typename T> struct BatchInst {
  Inst<T> I;
  FieldList inv, fwd;
  int nparts;   // partial sums of the stats pass
};

constexpr int BATCH_TX = 8;    // kx lines per CTA in the y/z passes of the generic class (FP32)
constexpr int BATCH_LYZ = 4;   // (y,z) lines per CTA in its x pass

// Kernel forms of a size class's passes, picked per pass by the server's autotuner:
//   y/z passes: line pairs on the packed FP32 pipe (8 kx lines a tile, n >= 64), or
//               one line per thread with 8 or 4 kx lines a tile;
//   x passes:   the register-fused pass (n = 64, 128), or the generic one with 4 or 2
//               (y,z) lines a CTA.
enum BatchYZForm : int { YZ_PAIR = 0, YZ_TX8 = 1, YZ_TX4 = 2, YZ_NFORMS = 3 };
enum BatchXForm : int { XF_FUSED = 0, XF_LYZ4 = 1, XF_LYZ2 = 2, XF_NFORMS = 3 };

// launch shape of one class's chain
struct ClassLaunch {
  int grid[BP_COUNT];
  int block[BP_COUNT];
  size_t smem[BP_COUNT];
  int form[BP_COUNT];   // BatchYZForm (y/z passes) or BatchXForm (x passes); 0 elsewhere
  int tile[BP_COUNT];   // kx lines of a work item (y/z passes), (y,z) lines (x passes), else 1
};

#define FFS_BATCH_LOOP(PH)                                                         \
  const int nwork = Tb->n[CI][PH];                                                 \
  const WorkItem* __restrict__ W = Tb->tab[CI][PH];                                \
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {                            \
    const WorkItem it = W[w];                                                      \
    const BatchInst<T>& BI = B[it.inst];

#define FFS_BATCH_END \
    __syncthreads();  \
  }

template <typename T, int TX, int CI = 0, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) kb_inv_z(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_INV_Z)
  b_inv_z<T, TX, N>(BI.I, BI.inv, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <typename T, int TX, int CI = 0, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) kb_inv_y(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_INV_Y)
  b_inv_y<T, TX, N>(BI.I, BI.inv, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <typename T, bool LES, int LYZ, int CI = 0, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) kb_x(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(LES ? BP_X_LES : BP_X)
  b_x_pass<T, LES, 0, LYZ, N>(BI.I, Blk{it.x, 0, 0, 0});
  FFS_BATCH_END
}
template <typename T, int TX, int CI = 0, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) kb_fwd_y(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_FWD_Y)
  b_fwd_y<T, TX, N>(BI.I, BI.fwd, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <typename T, int CI = 0>
__global__ void kb_scalar(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_SCALAR)
  b_scalar<T>(BI.I, 0, Blk{0, 0, 0, 1});
  FFS_BATCH_END
}
template <typename T, int CI = 0>
__global__ void kb_table(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_TABLE)
  b_etd_table<T>(BI.I, 0, Blk{it.x, 0, 0, it.y});
  FFS_BATCH_END
}
template <typename T, int TX, int CI = 0, int N = 0>
__global__ void __launch_bounds__(FFS_MAXT) kb_fwd_z(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_FWD_Z)
  b_fwd_z<T, TX, N>(BI.I, BI.fwd, 0, Blk{it.x, it.y, 0, 0});
  FFS_BATCH_END
}
template <typename T, int CI = 0>
__global__ void __launch_bounds__(256) kb_stats(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_STATS)
  b_stats<T>(BI.I, 0, Blk{it.x, 0, 0, it.y});
  b_spectra<T>(BI.I, 0, Blk{it.x, 0, 0, it.y});
  FFS_BATCH_END
}
template <typename T, int CI = 0>
__global__ void __launch_bounds__(256) kb_update(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_UPDATE)
  b_update<T>(BI.I, 0, Blk{it.x, 0, 0, it.y});
  FFS_BATCH_END
}
template <typename T, int CI = 0>
__global__ void __launch_bounds__(1024) kb_finalize(const BatchInst<T>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  FFS_BATCH_LOOP(BP_FIN)
  b_finalize<T>(BI.I, 0, BI.nparts, Blk{0, 0, 0, 1});
  FFS_BATCH_END
}

// Host side of one size class (ffs_batch_class.cuh, one translation unit per class):
// prepare() takes the form of each pass (null: the defaults), sets the kernels'
// shared-memory limits and computes the persistent grids; enqueue() launches the
// class's chain on a stream; launch() one pass (for the autotuner); forms() the bit
// mask of the forms a pass has.
struct ClassOps {
  int n;   // cubic side
  int (*prepare)(int device, int max_active, const int* form, ClassLaunch* L, std::string* err);
  void (*enqueue)(const ClassLaunch& L, cudaStream_t s, const BatchInst<float>* B, const BatchTables* T);
  void (*launch)(const ClassLaunch& L, int phase, cudaStream_t s, const BatchInst<float>* B, const BatchTables* T);
  unsigned (*forms)(int phase);
};
ClassOps batch_class_ops_32();
ClassOps batch_class_ops_48();
ClassOps batch_class_ops_64();
ClassOps batch_class_ops_96();
ClassOps batch_class_ops_128();

}  // namespace ffsgpu
