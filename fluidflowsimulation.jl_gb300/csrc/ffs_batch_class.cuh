// One size class of the batched step (cubic side N, class index CI): compile-time FFT
// plans, CTAs of exactly the threads each plan needs, every pass in each of its kernel
// forms (line pairs or one line per thread with 8 or 4 kx lines a tile for the y/z
// passes; for N = 64, 128 the register-fused x passes, else the generic x pass with 4
// or 2 (y,z) lines a CTA), so that the server's autotuner can pick one per pass. Included
// by one small translation unit per class, which defines batch_class_ops_<N>().
#pragma once
#include <mutex>
#include <string>

#include "../../include/ffs.h"
#include "ffs_batch.cuh"
#include "ffs_pairs.cuh"
#include "ffs_xfused.cuh"
#include "ffs_xles.cuh"

namespace ffsgpu {

template <int N, int CI>
__global__ void __launch_bounds__(XFused<N>::NT, XFusedCfg<N>::MINB)
kb_x_fused(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_X)
  b_x_fused<N>(BI.I, Blk{it.x, 0, 0, 0});
  FFS_BATCH_END
}

// the twelve-field fused x pass of LES runs (n = 64, 128; the batch serves no density)
template <int N, int CI>
__global__ void __launch_bounds__(XLes<N>::NT, XLesCfg<N>::MINB)
kb_x_les(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_X_LES)
  b_x_les<N, false>(BI.I, Blk{it.x, 0, 0, 0});
  FFS_BATCH_END
}

// y and z passes on line pairs (packed FP32; n >= 64, where a CTA is at least a warp)
template <int N, int CI>
__global__ void __launch_bounds__(PAIR_LP * ct_tpl<N>())
kb_inv_z2(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_INV_Z)
  b_inv_z2<N, PAIR_LP>(BI.I, BI.inv, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <int N, int CI>
__global__ void __launch_bounds__(PAIR_LP * ct_tpl<N>())
kb_inv_y2(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_INV_Y)
  b_inv_y2<N, PAIR_LP>(BI.I, BI.inv, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <int N, int CI>
__global__ void __launch_bounds__(PAIR_LP * ct_tpl<N>())
kb_fwd_y2(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_FWD_Y)
  b_fwd_y2<N, PAIR_LP>(BI.I, BI.fwd, Blk{it.x, it.y, it.z, 0});
  FFS_BATCH_END
}
template <int N, int CI>
__global__ void __launch_bounds__(PAIR_LP * ct_tpl<N>())
kb_fwd_z2(const BatchInst<float>* __restrict__ B, const BatchTables* __restrict__ Tb) {
  using T = float;
  FFS_BATCH_LOOP(BP_FWD_Z)
  b_fwd_z2<N, PAIR_LP>(BI.I, BI.fwd, 0, Blk{it.x, it.y, 0, 0});
  FFS_BATCH_END
}

template <int N, int CI>
struct BatchClass {
  static constexpr int tpl = ct_tpl<N>();
  static constexpr int nbuf = CtPlan<N>::np >= 3 ? 2 : 1;
  static constexpr bool FUSED = N == 64 || N == 128;    // velocity-only fused x pass
  static constexpr bool LESF = N == 64 || N == 128;     // LES fused x pass
  static constexpr bool PAIRF = N >= 64;                 // y/z passes on line pairs
  static constexpr int PT = 2 * PAIR_LP;                 // kx lines of a line-pair tile
  using KB = void (*)(const BatchInst<float>*, const BatchTables*);

  static bool yz(int ph) { return ph == BP_INV_Z || ph == BP_INV_Y || ph == BP_FWD_Y || ph == BP_FWD_Z; }
  static unsigned forms(int ph) {
    if (yz(ph)) return (PAIRF ? 1u << YZ_PAIR : 0u) | (1u << YZ_TX8) | (1u << YZ_TX4);
    if (ph == BP_X) return (FUSED ? 1u << XF_FUSED : 0u) | (1u << XF_LYZ4) | (1u << XF_LYZ2);
    if (ph == BP_X_LES) return (LESF ? 1u << XF_FUSED : 0u) | (1u << XF_LYZ4) | (1u << XF_LYZ2);
    return 1u;
  }
  static int default_form(int ph) {
    if (yz(ph)) return PAIRF ? YZ_PAIR : YZ_TX8;
    if (ph == BP_X) return FUSED ? XF_FUSED : XF_LYZ4;
    if (ph == BP_X_LES) return LESF ? XF_FUSED : XF_LYZ4;
    return 0;
  }

  // the kernel of a pass in a form (every batched kernel has the same signature)
  static KB kernel(int ph, int f) {
    switch (ph) {
      case BP_INV_Z:
        if constexpr (PAIRF) { if (f == YZ_PAIR) return kb_inv_z2<N, CI>; }
        return f == YZ_TX4 ? kb_inv_z<float, 4, CI, N> : kb_inv_z<float, 8, CI, N>;
      case BP_INV_Y:
        if constexpr (PAIRF) { if (f == YZ_PAIR) return kb_inv_y2<N, CI>; }
        return f == YZ_TX4 ? kb_inv_y<float, 4, CI, N> : kb_inv_y<float, 8, CI, N>;
      case BP_FWD_Y:
        if constexpr (PAIRF) { if (f == YZ_PAIR) return kb_fwd_y2<N, CI>; }
        return f == YZ_TX4 ? kb_fwd_y<float, 4, CI, N> : kb_fwd_y<float, 8, CI, N>;
      case BP_FWD_Z:
        if constexpr (PAIRF) { if (f == YZ_PAIR) return kb_fwd_z2<N, CI>; }
        return f == YZ_TX4 ? kb_fwd_z<float, 4, CI, N> : kb_fwd_z<float, 8, CI, N>;
      case BP_X:
        if constexpr (FUSED) { if (f == XF_FUSED) return kb_x_fused<N, CI>; }
        return f == XF_LYZ2 ? kb_x<float, false, 2, CI, N> : kb_x<float, false, 4, CI, N>;
      case BP_X_LES:
        if constexpr (LESF) { if (f == XF_FUSED) return kb_x_les<N, CI>; }
        return f == XF_LYZ2 ? kb_x<float, true, 2, CI, N> : kb_x<float, true, 4, CI, N>;
      case BP_SCALAR: return kb_scalar<float, CI>;
      case BP_TABLE: return kb_table<float, CI>;
      case BP_STATS: return kb_stats<float, CI>;
      case BP_UPDATE: return kb_update<float, CI>;
      default: return kb_finalize<float, CI>;
    }
  }

  // CTA size, dynamic shared memory and work-item tile of a pass in a form; a
  // compile-time plan needs exactly its threads (lines x threads per line, whole warps
  // for the x pass)
  static void shape(int ph, int f, int& block, size_t& smem, int& tile) {
    const size_t cb = sizeof(cplx<float>);
    const size_t mxp = (size_t)(N / 2 + 1) | 1;
    auto xs = [&](int nin, int lyz) {
      const size_t lin1 = (size_t)((nin + 1) / 2) * lyz + 1;
      return cb * ((size_t)srows(N) * lin1 + std::max((size_t)nin * lyz * mxp, (size_t)srows(N) * lin1));
    };
    constexpr int NP = PAIRF ? N : 64;
    block = 256; smem = 0; tile = 1;
    if (yz(ph)) {
      if (f == YZ_PAIR) {
        block = PAIR_LP * ct_tpl<NP>();
        smem = pair_smem<NP, PAIR_LP>() + (ph == BP_FWD_Z ? fwd_z2_aux_bytes<PT>(N) : 0);
        tile = PT;
      } else {
        const int tx = f == YZ_TX4 ? 4 : 8;
        // the forward z pass: three components together (and the i k.tau accumulators
        // for NZR <= N rows)
        block = (ph == BP_FWD_Z ? 3 : 1) * tx * tpl;
        smem = ph == BP_FWD_Z ? cb * ((size_t)3 * tx * srows(N) * nbuf + (size_t)4 * N * tx)
                              : (size_t)tx * srows(N) * cb * nbuf;
        tile = tx;
      }
      return;
    }
    if (ph == BP_X || ph == BP_X_LES) {
      const bool les = ph == BP_X_LES;
      if (f == XF_FUSED) {
        constexpr int NF = (N == 64 || N == 128) ? N : 64;
        block = les ? XLes<NF>::NT : XFused<NF>::NT;
        smem = les ? XLes<NF>::smem() : XFused<NF>::smem();
        tile = les ? XLes<NF>::LYZ : XFused<NF>::LYZ;
      } else {
        const int lyz = f == XF_LYZ2 ? 2 : 4, pin = les ? 6 : 3;
        block = ((pin * lyz * tpl + 31) / 32) * 32;
        smem = xs(les ? 11 : 6, lyz);
        tile = lyz;
      }
      return;
    }
    if (ph == BP_TABLE) block = 64;
    if (ph == BP_FIN) block = 1024;
  }

  // per-kernel limits are process-wide: only ever raised, under a lock
  static int attr(KB k, size_t bytes, std::string* err) {
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k);
    if (e == cudaSuccess && (int)bytes > fa.maxDynamicSharedSizeBytes)
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) { *err = std::string("batch class attribute: ") + cudaGetErrorString(e); return FFS_ECUDA; }
    return 0;
  }

  static int prepare(int device, int max_active, const int* form, ClassLaunch* L, std::string* err) {
    int sms = 0, maxs = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) {
      *err = "device attribute query failed";
      return FFS_ECUDA;
    }
    for (int ph = 0; ph < BP_COUNT; ++ph) {
      const int f = form ? form[ph] : default_form(ph);
      if (f < 0 || f > 2 || !((forms(ph) >> f) & 1u)) { *err = "batch class: no such kernel form"; return FFS_EINVAL; }
      L->form[ph] = f;
      shape(ph, f, L->block[ph], L->smem[ph], L->tile[ph]);
      const KB k = kernel(ph, f);
      cudaFuncAttributes fa;
      if (cudaFuncGetAttributes(&fa, k) != cudaSuccess || L->block[ph] > fa.maxThreadsPerBlock ||
          L->smem[ph] > (size_t)maxs) {
        *err = "batch class: form does not fit";
        return FFS_EUNSUPPORTED;
      }
      int rc;
      if (L->smem[ph] && (rc = attr(k, L->smem[ph], err))) return rc;
      int nb = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, L->block[ph], L->smem[ph]);
      if (e != cudaSuccess || nb < 1) { *err = "batch class kernel does not fit on an SM"; return FFS_EUNSUPPORTED; }
      // one-CTA-per-simulation passes need no more CTAs than simulations
      L->grid[ph] = (ph == BP_SCALAR || ph == BP_FIN) ? std::min(nb * sms, max_active) : nb * sms;
    }
    return 0;
  }

  static void launch(const ClassLaunch& L, int ph, cudaStream_t s, const BatchInst<float>* B, const BatchTables* T) {
    kernel(ph, L.form[ph])<<<L.grid[ph], L.block[ph], L.smem[ph], s>>>(B, T);
  }
  static void enqueue(const ClassLaunch& L, cudaStream_t s, const BatchInst<float>* B, const BatchTables* T) {
    for (int ph : {BP_INV_Z, BP_INV_Y, BP_X, BP_X_LES, BP_FWD_Y, BP_SCALAR, BP_TABLE, BP_FWD_Z, BP_STATS, BP_UPDATE,
                   BP_FIN})
      launch(L, ph, s, B, T);
  }
};

}  // namespace ffsgpu

#define FFS_DEFINE_BATCH_CLASS(NN, CI)                                                        \
  namespace ffsgpu {                                                                          \
  ClassOps batch_class_ops_##NN() {                                                           \
    return ClassOps{NN, &BatchClass<NN, CI>::prepare, &BatchClass<NN, CI>::enqueue,           \
                    &BatchClass<NN, CI>::launch, &BatchClass<NN, CI>::forms};                 \
  }                                                                                           \
  }
