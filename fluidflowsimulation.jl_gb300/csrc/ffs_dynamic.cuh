// The dynamic Smagorinsky models' extra passes (dynamic_smagorinsky.jl:3-217,
// dynamic_piomelli.jl:1-26, les_real_calc.jl:3-11): dynamicSmagorinsky, piomelliSmagorinsky
// (the previous coefficient extrapolated in time inside Sa), and either with the dynamic
// P tensor term (dynamicSandP, piomelliSandP: a second coefficient cp for D^2 Lie(S, W)).
//
// The model needs, at every grid point, the Germano coefficient
//   c = clamp(L:M / (2 M:M), -1, 1),  L = traceless(u^ u^ - (u u)^),
//   M = (D^2 + Dt^2) |S^| S^ - (D^2 |S| S)^,
// where ^ is the Gaussian test filter G = exp(-Dt^2 k^2 / 24) applied over the FULL
// spectrum (fullfourier!, not the dealiased one), and then c itself filtered the same way.
// So the step gains a second spectral layout: every mode kx 0..nx/2, all ky, all kz
// ("full" slots [slot][z][y][KXF], KXF = nx/2+1 padded to 8). The inverse z pass already
// produced u^ = G u and S^ = G S on the retained modes (prologue families 3 and 4).
//
//   k_dyn_x<0>:    u, S [, w] (retained)   -> physical -> Sa = D^2 |S| S, L = u u [, P] -> r2c, all kx
//   y/z/y passes:  full slots 0..nsa-1     -> forward y, [forward z, x G/N, inverse z], inverse y
//   k_dyn_x<1>:    u^, S^ [, w^] (retained), Sa~, L~ [, P~] (full) -> physical -> c [, cp]
//                  -> r2c into full slot nsa [, nsa+1]
//   y/z/y passes:  those slots             -> the averaged coefficients
//   k_inv_x_phys:  those slots             -> physical c [, cp], read by the x pass
//
// One (y,z) line per CTA in the x kernels; the shared memory holds every input line of
// that (y,z) line (19 fields in the coefficient pass), which bounds nx (checked at create).
#pragma once
#include "ffs_kernels.cuh"

namespace ffsgpu {

template <typename T> struct DynFull {
  cplx<T>* fy;        // [slot][z][y][kxf]: x-spectral fields over the full spectrum
  long long fys;      // slot stride
  int kxf;            // row length (>= nx/2 + 1, a multiple of 8)
  int gslot0;         // first wy slot of the test-filtered u^ (3), S^ (5) [, w^ (3)]
  int nsa;            // full slots of Sa, L [, P]; the coefficient c [and cp] follow
};

// Full slots: Sa (5: xx xy xz yy yz), L (6: xx xy xz yy yz zz), with the dynamic P tensor
// P (5), then c and cp.
constexpr int DYN_NSA = 11;
constexpr int DYN_NSA_P = 16;
constexpr int DYN_NSLOTS = 12;
constexpr int DYN_NSLOTS_P = 18;

template <int STAGE, bool DP> struct DynX {
  static constexpr int NRET = DP ? 11 : 8;                        // stage 1: u^, S^ [, w^]
  static constexpr int NIN = STAGE == 0 ? (DP ? 11 : 8) : NRET + (DP ? 16 : 11);
  static constexpr int LIN = (NIN + 1) / 2;
  static constexpr int NOUT = STAGE == 0 ? (DP ? DYN_NSA_P : DYN_NSA) : (DP ? 2 : 1);
  static constexpr int LOUT = (NOUT + 1) / 2;
  static constexpr int LS = (LIN > LOUT ? LIN : LOUT) | 1;   // odd line stride
  static size_t smem(int nx, size_t cb) { return 2 * (size_t)srows(nx) * LS * cb; }
};

// Lie(S, W) = S W - W S of the traceless symmetric S (xx, xy, xz, yy, yz) and
// W = AntiSymTen(w/2), the cross-product matrix of w/2; symmetric and traceless: its
// five stored components
template <typename T>
__device__ __forceinline__ void lie_sw(T xx, T xy, T xz, T yy, T yz, T wx, T wy, T wz, T* o) {
  const T zz = -xx - yy;
  const T S[3][3] = {{xx, xy, xz}, {xy, yy, yz}, {xz, yz, zz}};
  const T p = T(0.5) * wx, q = T(0.5) * wy, r = T(0.5) * wz;
  const T W[3][3] = {{T(0), -r, q}, {r, T(0), -p}, {-q, p, T(0)}};
  T L[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T a = T(0), b = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) { a += S[i][k] * W[k][j]; b += W[i][k] * S[k][j]; }
      L[i][j] = a - b;
    }
  o[0] = L[0][0]; o[1] = L[0][1]; o[2] = L[0][2]; o[3] = L[1][1]; o[4] = L[1][2];
}

// (t + L) : M / (M:M) of the traceless t, M (5 components each) and the traceless L (6)
template <typename T>
__device__ __forceinline__ T ddot_norm(const T* t, const T* M, const T* L6) {
  const T mzz = -M[0] - M[3], tzz = -t[0] - t[3];
  const T mm = M[0] * M[0] + M[3] * M[3] + mzz * mzz + T(2) * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
  return (t[0] + L6[0]) * (M[0] / mm) + (t[3] + L6[3]) * (M[3] / mm) + (tzz + L6[5]) * (mzz / mm) +
         T(2) * ((t[1] + L6[1]) * (M[1] / mm) + (t[2] + L6[2]) * (M[2] / mm) + (t[4] + L6[4]) * (M[4] / mm));
}

// max(lo, min(hi, v)) with Julia's NaN propagation
template <typename T> __device__ __forceinline__ T clampn(T v, T lo, T hi) {
  return isnan(v) ? v : (v > hi ? hi : (v < lo ? lo : v));
}

// calc_cstar! (dynamic_smagorinsky.jl:9-35, dynamic_piomelli.jl:1-11): the coefficient
// ratio dt/dtm1 of this step (dt: the current one; set_dt! runs after these passes)
__device__ __forceinline__ double cstar_ratio(double dt, double dtm1) {
  const double dtf = dt == 0.0 ? 1.0 : dt, dtm1f = dtm1 == 0.0 ? dtf : dtm1;
  return dtf / dtm1f;
}

template <typename T, int STAGE, bool DP>
__global__ void __launch_bounds__(256) k_dyn_x(Inst<T> I, DynFull<T> D) {
  using X = DynX<STAGE, DP>;
  constexpr int NIN = X::NIN, LIN = X::LIN, NOUT = X::NOUT, LOUT = X::LOUT, LS = X::LS, NRET = X::NRET;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = I.nx, nxh = I.nxh;
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + (size_t)srows(n) * LS;
  const long long g = blockIdx.x;   // (y,z) line z * ny + y
  const long long plane = (long long)I.nx * I.ny * I.nz;

  // input field f of this line and the count of kx it holds
  auto src = [&](int f, int& M) -> const cplx<T>* {
    if (STAGE == 0) {   // u (slots 0..2), S (slots 6..10) [, w (slots 3..5)]
      M = I.Mx;
      const int slot = f < 3 ? f : (f < 8 ? f + 3 : f - 5);
      return I.wy + (long long)slot * I.wys + g * I.KXP;
    }
    if (f < NRET) {     // u^, S^ [, w^]
      M = I.Mx;
      return I.wy + (long long)(D.gslot0 + f) * I.wys + g * I.KXP;
    }
    M = nxh;            // Sa~, L~ [, P~]
    return D.fy + (long long)(f - NRET) * D.fys + g * D.kxf;
  };
  // c2r, two real fields per complex line (brfft: unnormalised)
  auto ldi = [&](int l, int j) -> cplx<T> {
    const bool cj = 2 * j > n;
    const int k = cj ? n - j : j;
    const int fa = 2 * l, fb = 2 * l + 1;
    int Ma = 0, Mb = 0;
    const cplx<T>* pa = src(fa, Ma);
    cplx<T> A = k < Ma ? pa[k] : mk(T(0), T(0));
    cplx<T> B = mk(T(0), T(0));
    if (fb < NIN) {
      const cplx<T>* pb = src(fb, Mb);
      if (k < Mb) B = pb[k];
    }
    if (k == 0 || 2 * k == n) { A.y = T(0); B.y = T(0); }
    if (cj) { A.y = -A.y; B.y = -B.y; }
    return mk(A.x - B.y, A.y + B.x);
  };
  cplx<T>* ri = fft_result_buffer(I.px, s0, s1);
  auto sti = [&](int l, int j, cplx<T> v) { ri[sidx(j, l, LS)] = v; };
  fft_lines<+1, LIN, T>(I.px, s0, s1, LS, I.twx, ldi, sti);

  // pointwise: inputs from ri, outputs to s1 at the same row (same thread)
  const T d2 = T(I.les_d2);
  // time-extrapolated coefficients: c* = c + (dt/dtm1)(c - cm1), then cm1 := c (cm1 := c
  // first at iteration 0); piomelliSmagorinsky's c and piomelliSandP's cp
  double rpi = 0.0, rpp = 0.0;
  bool first = false;
  if (STAGE == 0) {
    rpi = cstar_ratio(I.st->dt, I.st->dyn_dtm1);
    rpp = cstar_ratio(I.st->dt, I.st->dyn_dtpm1);
    first = I.st->iteration == 0;
  }
  if (STAGE == 1 && blockIdx.x == 0 && threadIdx.x == 0) {
    if (I.piom) I.st->dyn_dtm1 = I.st->dt;
    if (I.dynp == 2) I.st->dyn_dtpm1 = I.st->dt;
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const cplx<T>* row = ri + sidx(j, 0, LS);
    T f[2 * LIN];
#pragma unroll
    for (int p = 0; p < LIN; ++p) { const cplx<T> v = row[p]; f[2 * p] = v.x; f[2 * p + 1] = v.y; }
    T o[2 * LOUT];
#pragma unroll
    for (int r = 0; r < 2 * LOUT; ++r) o[r] = T(0);
    const long long pi = g * n + j;   // physical index [z][y][x]
    if (STAGE == 0) {
      // realspace_dynamic_les_calculation! (dynamic_smagorinsky.jl:42-77): Sa = D^2 |S| S
      // (2 c* D^2 |S| S for piomelliSmagorinsky), L = u u [, P = (cp*) D^2 Lie(S, W)]
      const T ux = f[0], uy = f[1], uz = f[2];
      const T xx = f[3], xy = f[4], xz = f[5], yy = f[6], yz = f[7], zz = -xx - yy;
      const T nrm = sqrt(xx * xx + yy * yy + zz * zz + T(2) * (xy * xy + xz * xz + yz * yz));
      T a = d2 * nrm;
      if (I.piom) {
        const double cv = I.dyn_c[pi], cm = first ? cv : I.dyn_cm1[pi];
        const double cs = rpi * (cv - cm) + cv;
        I.dyn_cm1[pi] = cv;
        a = T(2) * T(cs) * d2 * nrm;
      }
      o[0] = a * xx; o[1] = a * xy; o[2] = a * xz; o[3] = a * yy; o[4] = a * yz;
      o[5] = ux * ux; o[6] = ux * uy; o[7] = ux * uz; o[8] = uy * uy; o[9] = uy * uz; o[10] = uz * uz;
      if constexpr (DP) {
        T lie[5];
        lie_sw<T>(xx, xy, xz, yy, yz, f[8], f[9], f[10], lie);
        T b = d2;
        if (I.dynp == 2) {
          const double cv = I.dyn_c[plane + pi], cm = first ? cv : I.dyn_cpm1[pi];
          const double cs = rpp * (cv - cm) + cv;
          I.dyn_cpm1[pi] = cv;
          b = T(cs) * d2;
        }
#pragma unroll
        for (int q = 0; q < 5; ++q) o[11 + q] = b * lie[q];
      }
    } else {
      // coefficient_les_calculation! (dynamic_smagorinsky.jl:118-205)
      const T a = f[0], b = f[1], c = f[2];
      const T* Sh = f + 3;                 // S^
      const T* Sa = f + NRET;              // Sa~
      const T* Lf = f + NRET + 5;          // (u u)~
      T L6[6] = {a * a - Lf[0], a * b - Lf[1], a * c - Lf[2], b * b - Lf[3], b * c - Lf[4], c * c - Lf[5]};
      const T tr = (L6[0] + L6[3] + L6[5]) / T(3);
      L6[0] -= tr; L6[3] -= tr; L6[5] -= tr;
      const T hzz = -Sh[0] - Sh[3];
      const T nh = sqrt(Sh[0] * Sh[0] + Sh[3] * Sh[3] + hzz * hzz + T(2) * (Sh[1] * Sh[1] + Sh[2] * Sh[2] + Sh[4] * Sh[4]));
      const T dsum = T(I.dyn_d2h + I.les_d2);
      T tau[5];   // tau^ of the piomelli forms: Sa~ (+ P~ with piomelliSandP)
#pragma unroll
      for (int q = 0; q < 5; ++q) tau[q] = Sa[q];
      if constexpr (DP) {
        if (I.dynp == 2) {
#pragma unroll
          for (int q = 0; q < 5; ++q) tau[q] = Sa[q] + f[NRET + 11 + q];
        }
      }
      T cv;
      if (I.piom) {
        // c = (tau^ + L) : M / (M:M), M = 2 (D^^2 + D^2) |S^| S^
        const T s = T(2) * dsum * nh;
        const T M[5] = {s * Sh[0], s * Sh[1], s * Sh[2], s * Sh[3], s * Sh[4]};
        cv = ddot_norm<T>(tau, M, L6);
      } else {
        // c = L:M / (2 M:M), M = (D^^2 + D^2) |S^| S^ - Sa~
        const T s = dsum * nh;
        const T mxx = s * Sh[0] - Sa[0], mxy = s * Sh[1] - Sa[1], mxz = s * Sh[2] - Sa[2];
        const T myy = s * Sh[3] - Sa[3], myz = s * Sh[4] - Sa[4], mzz = -mxx - myy;
        const T lm = L6[0] * mxx + L6[3] * myy + L6[5] * mzz + T(2) * (L6[1] * mxy + L6[2] * mxz + L6[4] * myz);
        const T mm = mxx * mxx + myy * myy + mzz * mzz + T(2) * (mxy * mxy + mxz * mxz + myz * myz);
        cv = T(0.5) * (lm / mm);
      }
      o[0] = clampn(cv, T(-1), T(1));
      if constexpr (DP) {
        // cp from P^ = Lie(S^, AntiSymTen(w^/2)) (dynamic_smagorinsky.jl:188-203)
        T Ph[5];
        lie_sw<T>(Sh[0], Sh[1], Sh[2], Sh[3], Sh[4], f[8], f[9], f[10], Ph);
        const T* Pf = f + NRET + 11;       // P~
        T cp;
        if (I.dynp == 1) {   // Mp = (D^^2 + D^2) P^ - P~, cp = L:Mp / Mp:Mp
          T Mp[5];
#pragma unroll
          for (int q = 0; q < 5; ++q) Mp[q] = dsum * Ph[q] - Pf[q];
          const T mzz = -Mp[0] - Mp[3];
          const T lm = L6[0] * Mp[0] + L6[3] * Mp[3] + L6[5] * mzz + T(2) * (L6[1] * Mp[1] + L6[2] * Mp[2] + L6[4] * Mp[4]);
          const T mm = Mp[0] * Mp[0] + Mp[3] * Mp[3] + mzz * mzz + T(2) * (Mp[1] * Mp[1] + Mp[2] * Mp[2] + Mp[4] * Mp[4]);
          cp = lm / mm;
        } else {             // Mp = (D^^2 + D^2) P^, cp = (tau^ + L) : Mp / Mp:Mp
          T Mp[5], tp[5];
#pragma unroll
          for (int q = 0; q < 5; ++q) { Mp[q] = dsum * Ph[q]; tp[q] = I.piom ? tau[q] : Pf[q]; }
          cp = ddot_norm<T>(tp, Mp, L6);
        }
        o[1] = clampn(cp, T(-1), T(1));
      }
    }
    cplx<T>* orow = s1 + sidx(j, 0, LS);
#pragma unroll
    for (int r = 0; r < LOUT; ++r) orow[r] = mk(o[2 * r], o[2 * r + 1]);
  }
  __syncthreads();

  // r2c (rfft!: unnormalised; 1/N is applied with the filter) over every kx
  cplx<T>* rf = fft_result_buffer(I.px, s0, s1);
  auto ldf = [&](int l, int j) -> cplx<T> { return s1[sidx(j, l, LS)]; };
  auto stf = [&](int l, int j, cplx<T> v) { rf[sidx(j, l, LS)] = v; };
  fft_lines<-1, LOUT, T>(I.px, s0, s1, LS, I.twx, ldf, stf);
  const int slot0 = STAGE == 0 ? 0 : D.nsa;
  for (int e = threadIdx.x; e < LOUT * D.kxf; e += blockDim.x) {
    const int k = e % D.kxf, r = e / D.kxf;
    cplx<T> A = mk(T(0), T(0)), B = mk(T(0), T(0));
    if (k < nxh) {
      const cplx<T> zk = rf[sidx(k, r, LS)];
      const cplx<T> zm = rf[sidx(k == 0 ? 0 : n - k, r, LS)];
      A = mk(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
      B = mk(T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x));
    }
    D.fy[(long long)(slot0 + 2 * r) * D.fys + g * D.kxf + k] = A;
    if (2 * r + 1 < NOUT) D.fy[(long long)(slot0 + 2 * r + 1) * D.fys + g * D.kxf + k] = B;
  }
}

// fill n doubles with v (the piomelli coefficient's initial value)
static __global__ void k_dyn_fill(double* p, long long n, double v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// Test filter along z on the full layout (J: the full-spectrum instance, wz = [slot][z][y][kxf]):
// forward z, times G(k) / (nx ny nz) (fullmyscale! and the Gaussfilter multiply of
// fourierspace_dynamic_les_calculation! / average_c!), inverse z, in place.
// grid (nfields, kxf / TXL, ny); block TXL * tpl_z; shared 2 * srows(nz) * TXL.
template <typename T, int TXL>
__global__ void __launch_bounds__(FFS_MAXT) k_dyn_zfilter(Inst<T> J, int slot0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + (size_t)srows(J.nz) * TXL;
  const int fi = blockIdx.x, kx0 = blockIdx.y * TXL, y = blockIdx.z;
  const long long rs = (long long)J.ny * J.KXP;
  cplx<T>* col = J.wz + (long long)(slot0 + fi) * J.wzs + (long long)y * J.KXP + kx0;
  const T ky = kval(y < J.ny / 2 ? y : y - J.ny, J.Ly_t, J.iLy_t);
  const T aux = T(-J.dyn_d2h / 24.0), sc = T(J.inv_n);
  auto ld = [&](int l, int z) -> cplx<T> { return col[(long long)z * rs + l]; };
  // the last pass writes the positions it read: its result may go to s1 in every plan
  auto st = [&](int l, int z, cplx<T> v) {
    const T kx = kval(kx0 + l, J.Lx_t, J.iLx_t), kz = kval(z < J.nz / 2 ? z : z - J.nz, J.Lz_t, J.iLz_t);
    const T gk = exp(aux * (kx * kx + (ky * ky + kz * kz)));
    s1[sidx(z, l, TXL)] = scl(scl(v, sc), gk);
  };
  fft_lines<-1, TXL, T>(J.pz, s0, s1, TXL, J.twz, ld, st);
  auto ld2 = [&](int l, int z) -> cplx<T> { return s1[sidx(z, l, TXL)]; };
  auto st2 = [&](int l, int z, cplx<T> v) { col[(long long)z * rs + l] = v; };
  fft_lines<+1, TXL, T>(J.pz, s0, s1, TXL, J.twz, ld2, st2);
}

}  // namespace ffsgpu
