// One size class of the batched step (cubic side N, class index CI): compile-time FFT
// plans, CTAs of exactly the threads each plan needs, and for N = 64, 128 the
// register-fused x passes of velocity-only and LES runs. Included by one small translation unit per class, which
// defines batch_class_ops_<N>().
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
  static constexpr int TX = BATCH_TX, LYZ = BATCH_LYZ;
  static constexpr int tpl = ct_tpl<N>();
  static constexpr int nbuf = CtPlan<N>::np >= 3 ? 2 : 1;
  static constexpr bool FUSED = N == 64 || N == 128;    // velocity-only fused x pass
  static constexpr bool LESF = N == 64 || N == 128;     // LES fused x pass
  static constexpr bool PAIRF = N >= 64;                 // y/z passes on line pairs
  static_assert(2 * PAIR_LP == TX, "line pairs cover the TX lines of a tile");

  // per-kernel limits are process-wide: only ever raised, under a lock
  template <typename K> static int attr(K k, size_t bytes, std::string* err) {
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k);
    if (e == cudaSuccess && (int)bytes > fa.maxDynamicSharedSizeBytes)
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) { *err = std::string("batch class attribute: ") + cudaGetErrorString(e); return FFS_ECUDA; }
    return 0;
  }
  template <typename K> static int occ(K k, ClassLaunch* L, int ph, int sms, int cap, std::string* err) {
    int nb = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, L->block[ph], L->smem[ph]);
    if (e != cudaSuccess || nb < 1) { *err = "batch class kernel does not fit on an SM"; return FFS_EUNSUPPORTED; }
    L->grid[ph] = std::min(nb * sms, cap);
    return 0;
  }

  static int prepare(int device, int max_active, ClassLaunch* L, std::string* err) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
      *err = "device attribute query failed";
      return FFS_ECUDA;
    }
    const size_t cb = sizeof(cplx<float>);
    const size_t mxp = (size_t)(N / 2 + 1) | 1;
    auto xs = [&](int nin) {
      const size_t lin1 = (size_t)((nin + 1) / 2) * LYZ + 1;
      return cb * ((size_t)srows(N) * lin1 + std::max((size_t)nin * LYZ * mxp, (size_t)srows(N) * lin1));
    };
    L->block[BP_INV_Z] = L->block[BP_INV_Y] = L->block[BP_FWD_Y] = TX * tpl;
    L->smem[BP_INV_Z] = L->smem[BP_INV_Y] = L->smem[BP_FWD_Y] = (size_t)TX * srows(N) * cb * nbuf;
    if (FUSED) { L->block[BP_X] = XFused<FUSED ? N : 128>::NT; L->smem[BP_X] = XFused<FUSED ? N : 128>::smem(); }
    else { L->block[BP_X] = ((3 * LYZ * tpl + 31) / 32) * 32; L->smem[BP_X] = xs(6); }
    if (LESF) { L->block[BP_X_LES] = XLes<LESF ? N : 64>::NT; L->smem[BP_X_LES] = XLes<LESF ? N : 64>::smem(); }
    else { L->block[BP_X_LES] = 6 * LYZ * tpl; L->smem[BP_X_LES] = xs(11); }
    L->block[BP_FWD_Z] = 3 * TX * tpl;
    L->smem[BP_FWD_Z] = cb * ((size_t)3 * TX * srows(N) * nbuf + (size_t)4 * N * TX);
    if (PAIRF) {   // (the i k.tau accumulators for NZR <= N rows)
      constexpr int NP = PAIRF ? N : 64;
      L->block[BP_FWD_Y] = L->block[BP_FWD_Z] = L->block[BP_INV_Z] = L->block[BP_INV_Y] = PAIR_LP * ct_tpl<NP>();
      L->smem[BP_FWD_Y] = L->smem[BP_INV_Z] = L->smem[BP_INV_Y] = pair_smem<NP, PAIR_LP>();
      L->smem[BP_FWD_Z] = pair_smem<NP, PAIR_LP>() + fwd_z2_aux_bytes<TX>(N);
    }
    L->block[BP_SCALAR] = 256; L->block[BP_TABLE] = 64; L->block[BP_STATS] = 256; L->block[BP_UPDATE] = 256;
    L->block[BP_FIN] = 1024;
    L->smem[BP_SCALAR] = L->smem[BP_TABLE] = L->smem[BP_STATS] = L->smem[BP_UPDATE] = L->smem[BP_FIN] = 0;
    int rc;
    const int big = 1 << 30;
    if ((rc = PAIRF ? 0 : attr(kb_inv_z<float, TX, CI, N>, L->smem[BP_INV_Z], err)) ||
        (rc = PAIRF ? 0 : attr(kb_inv_y<float, TX, CI, N>, L->smem[BP_INV_Y], err)) ||
        (rc = PAIRF ? 0 : attr(kb_fwd_y<float, TX, CI, N>, L->smem[BP_FWD_Y], err)) ||
        (rc = PAIRF ? 0 : attr(kb_fwd_z<float, TX, CI, N>, L->smem[BP_FWD_Z], err)))
      return rc;
    if constexpr (PAIRF) {
      if ((rc = attr(kb_fwd_y2<N, CI>, L->smem[BP_FWD_Y], err)) || (rc = attr(kb_fwd_z2<N, CI>, L->smem[BP_FWD_Z], err)) ||
          (rc = occ(kb_fwd_y2<N, CI>, L, BP_FWD_Y, sms, big, err)) || (rc = occ(kb_fwd_z2<N, CI>, L, BP_FWD_Z, sms, big, err)) ||
          (rc = attr(kb_inv_z2<N, CI>, L->smem[BP_INV_Z], err)) || (rc = attr(kb_inv_y2<N, CI>, L->smem[BP_INV_Y], err)) ||
          (rc = occ(kb_inv_z2<N, CI>, L, BP_INV_Z, sms, big, err)) || (rc = occ(kb_inv_y2<N, CI>, L, BP_INV_Y, sms, big, err)))
        return rc;
    } else {
      if ((rc = occ(kb_fwd_y<float, TX, CI, N>, L, BP_FWD_Y, sms, big, err)) ||
          (rc = occ(kb_fwd_z<float, TX, CI, N>, L, BP_FWD_Z, sms, big, err)) ||
          (rc = occ(kb_inv_z<float, TX, CI, N>, L, BP_INV_Z, sms, big, err)) ||
          (rc = occ(kb_inv_y<float, TX, CI, N>, L, BP_INV_Y, sms, big, err)))
        return rc;
    }
    if constexpr (LESF) {
      if ((rc = attr(kb_x_les<N, CI>, L->smem[BP_X_LES], err))) return rc;
      if ((rc = occ(kb_x_les<N, CI>, L, BP_X_LES, sms, big, err))) return rc;
    } else {
      if ((rc = attr(kb_x<float, true, LYZ, CI, N>, L->smem[BP_X_LES], err))) return rc;
      if ((rc = occ(kb_x<float, true, LYZ, CI, N>, L, BP_X_LES, sms, big, err))) return rc;
    }
    if constexpr (FUSED) {
      if ((rc = attr(kb_x_fused<N, CI>, L->smem[BP_X], err))) return rc;
      if ((rc = occ(kb_x_fused<N, CI>, L, BP_X, sms, big, err))) return rc;
    } else {
      if ((rc = attr(kb_x<float, false, LYZ, CI, N>, L->smem[BP_X], err))) return rc;
      if ((rc = occ(kb_x<float, false, LYZ, CI, N>, L, BP_X, sms, big, err))) return rc;
    }
    if ((rc = occ(kb_scalar<float, CI>, L, BP_SCALAR, sms, max_active, err)) ||
        (rc = occ(kb_table<float, CI>, L, BP_TABLE, sms, big, err)) ||
        (rc = occ(kb_stats<float, CI>, L, BP_STATS, sms, big, err)) ||
        (rc = occ(kb_update<float, CI>, L, BP_UPDATE, sms, big, err)) ||
        (rc = occ(kb_finalize<float, CI>, L, BP_FIN, sms, max_active, err)))
      return rc;
    return 0;
  }

  static void enqueue(const ClassLaunch& L, cudaStream_t s, const BatchInst<float>* B, const BatchTables* T) {
#define FFS_CL(PH) L.grid[PH], L.block[PH], L.smem[PH], s
    if constexpr (PAIRF) {
      kb_inv_z2<N, CI><<<FFS_CL(BP_INV_Z)>>>(B, T);
      kb_inv_y2<N, CI><<<FFS_CL(BP_INV_Y)>>>(B, T);
    } else {
      kb_inv_z<float, TX, CI, N><<<FFS_CL(BP_INV_Z)>>>(B, T);
      kb_inv_y<float, TX, CI, N><<<FFS_CL(BP_INV_Y)>>>(B, T);
    }
    if constexpr (FUSED) kb_x_fused<N, CI><<<FFS_CL(BP_X)>>>(B, T);
    else kb_x<float, false, LYZ, CI, N><<<FFS_CL(BP_X)>>>(B, T);
    if constexpr (LESF) kb_x_les<N, CI><<<FFS_CL(BP_X_LES)>>>(B, T);
    else kb_x<float, true, LYZ, CI, N><<<FFS_CL(BP_X_LES)>>>(B, T);
    if constexpr (PAIRF) kb_fwd_y2<N, CI><<<FFS_CL(BP_FWD_Y)>>>(B, T);
    else kb_fwd_y<float, TX, CI, N><<<FFS_CL(BP_FWD_Y)>>>(B, T);
    kb_scalar<float, CI><<<FFS_CL(BP_SCALAR)>>>(B, T);
    kb_table<float, CI><<<FFS_CL(BP_TABLE)>>>(B, T);
    if constexpr (PAIRF) kb_fwd_z2<N, CI><<<FFS_CL(BP_FWD_Z)>>>(B, T);
    else kb_fwd_z<float, TX, CI, N><<<FFS_CL(BP_FWD_Z)>>>(B, T);
    kb_stats<float, CI><<<FFS_CL(BP_STATS)>>>(B, T);
    kb_update<float, CI><<<FFS_CL(BP_UPDATE)>>>(B, T);
    kb_finalize<float, CI><<<FFS_CL(BP_FIN)>>>(B, T);
#undef FFS_CL
  }
};

}  // namespace ffsgpu

#define FFS_DEFINE_BATCH_CLASS(NN, CI)                                                        \
  namespace ffsgpu {                                                                          \
  ClassOps batch_class_ops_##NN() {                                                           \
    return ClassOps{NN, &BatchClass<NN, CI>::prepare, &BatchClass<NN, CI>::enqueue};          \
  }                                                                                           \
  }
