// The dynamic Smagorinsky model's extra passes (dynamic_smagorinsky.jl:3-217,
// dynamic_piomelli.jl:13-26, les_real_calc.jl:3-11).
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
//   k_dyn_x<0>:    u, S (retained)         -> physical -> Sa = D^2 |S| S, L = u u -> r2c, all kx
//   y/z/y passes:  full slots 0..10        -> forward y, [forward z, x G/N, inverse z], inverse y
//   k_dyn_x<1>:    u^, S^ (retained), Sa^, L^ (full) -> physical -> c -> r2c into full slot 11
//   y/z/y passes:  full slot 11            -> the averaged coefficient
//   k_inv_x_phys:  full slot 11            -> physical c, read by the x pass (nu_t)
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
  int gslot0;         // first wy slot of the test-filtered u^ (3), S^ (5)
};

// Slots of the full layout.
constexpr int DYN_NSA = 11;   // Sa (5: xx xy xz yy yz), then L (6: xx xy xz yy yz zz)
constexpr int DYN_SLOT_C = 11;
constexpr int DYN_NSLOTS = 12;

template <int STAGE> struct DynX {
  static constexpr int NIN = STAGE == 0 ? 8 : 19;
  static constexpr int LIN = (NIN + 1) / 2;
  static constexpr int NOUT = STAGE == 0 ? DYN_NSA : 1;
  static constexpr int LOUT = (NOUT + 1) / 2;
  static constexpr int LS = (LIN > LOUT ? LIN : LOUT) | 1;   // odd line stride
  static size_t smem(int nx, size_t cb) { return 2 * (size_t)srows(nx) * LS * cb; }
};

template <typename T, int STAGE>
__global__ void __launch_bounds__(256) k_dyn_x(Inst<T> I, DynFull<T> D) {
  using X = DynX<STAGE>;
  constexpr int NIN = X::NIN, LIN = X::LIN, NOUT = X::NOUT, LOUT = X::LOUT, LS = X::LS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = I.nx, nxh = I.nxh;
  cplx<T>* s0 = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s1 = s0 + (size_t)srows(n) * LS;
  const long long g = blockIdx.x;   // (y,z) line z * ny + y

  // input field f of this line and the count of kx it holds
  auto src = [&](int f, int& M) -> const cplx<T>* {
    if (STAGE == 0) {   // u (slots 0..2), S (slots 6..10)
      M = I.Mx;
      return I.wy + (long long)(f < 3 ? f : f + 3) * I.wys + g * I.KXP;
    }
    if (f < 8) {        // u^, S^
      M = I.Mx;
      return I.wy + (long long)(D.gslot0 + f) * I.wys + g * I.KXP;
    }
    M = nxh;            // Sa^, L^
    return D.fy + (long long)(f - 8) * D.fys + g * D.kxf;
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
  // piomelliSmagorinsky (calc_cstar!, dynamic_smagorinsky.jl:9-19, dynamic_piomelli.jl:1-11):
  // c* = c + (dt/dtm1)(c - cm1) from the last averaged c, then cm1 := c (cm1 := c first at
  // iteration 0); dt is the step's current dt (set_dt! runs after this pass)
  double rpi = 0.0;
  bool first = false;
  if (STAGE == 0 && I.piom) {
    const double dt = I.st->dt, dtm1 = I.st->dyn_dtm1;
    const double dtf = dt == 0.0 ? 1.0 : dt, dtm1f = dtm1 == 0.0 ? dtf : dtm1;
    rpi = dtf / dtm1f;
    first = I.st->iteration == 0;
  }
  if (STAGE == 1 && I.piom && blockIdx.x == 0 && threadIdx.x == 0) I.st->dyn_dtm1 = I.st->dt;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const cplx<T>* row = ri + sidx(j, 0, LS);
    T f[2 * LIN];
#pragma unroll
    for (int p = 0; p < LIN; ++p) { const cplx<T> v = row[p]; f[2 * p] = v.x; f[2 * p + 1] = v.y; }
    T o[2 * LOUT];
#pragma unroll
    for (int r = 0; r < 2 * LOUT; ++r) o[r] = T(0);
    if (STAGE == 0) {
      // realspace_dynamic_les_calculation! (dynamic_smagorinsky.jl:66-72): Sa = D^2 |S| S, L = u u
      const T ux = f[0], uy = f[1], uz = f[2];
      const T xx = f[3], xy = f[4], xz = f[5], yy = f[6], yz = f[7], zz = -xx - yy;
      const T nrm = sqrt(xx * xx + yy * yy + zz * zz + T(2) * (xy * xy + xz * xz + yz * yz));
      T a = d2 * nrm;
      if (I.piom) {   // Sa = 2 c* D^2 |S| S
        const long long pi = g * n + j;
        const double cv = I.dyn_c[pi], cm = first ? cv : I.dyn_cm1[pi];
        const double cs = rpi * (cv - cm) + cv;
        I.dyn_cm1[pi] = cv;
        a = T(2) * T(cs) * d2 * nrm;
      }
      o[0] = a * xx; o[1] = a * xy; o[2] = a * xz; o[3] = a * yy; o[4] = a * yz;
      o[5] = ux * ux; o[6] = ux * uy; o[7] = ux * uz; o[8] = uy * uy; o[9] = uy * uz; o[10] = uz * uz;
    } else {
      // coefficient_les_calculation! (dynamic_smagorinsky.jl:162-172)
      const T a = f[0], b = f[1], c = f[2];
      const T hxx = f[3], hxy = f[4], hxz = f[5], hyy = f[6], hyz = f[7], hzz = -hxx - hyy;
      T l0 = a * a - f[13], l1 = a * b - f[14], l2 = a * c - f[15];
      T l3 = b * b - f[16], l4 = b * c - f[17], l5 = c * c - f[18];
      const T tr = (l0 + l3 + l5) / T(3);
      l0 -= tr; l3 -= tr; l5 -= tr;
      const T nh = sqrt(hxx * hxx + hyy * hyy + hzz * hzz + T(2) * (hxy * hxy + hxz * hxz + hyz * hyz));
      T cv;
      if (I.piom) {
        // c = (tau^ + L) : M / (M:M), M = 2 (D^^2 + D^2) |S^| S^ (dynamic_smagorinsky.jl:174-185)
        const T s = T(2) * T(I.dyn_d2h + I.les_d2) * nh;
        const T mxx = s * hxx, mxy = s * hxy, mxz = s * hxz, myy = s * hyy, myz = s * hyz, mzz = -mxx - myy;
        const T mm = mxx * mxx + myy * myy + mzz * mzz + T(2) * (mxy * mxy + mxz * mxz + myz * myz);
        const T txx = f[8], txy = f[9], txz = f[10], tyy = f[11], tyz = f[12], tzz = -txx - tyy;
        cv = (txx + l0) * (mxx / mm) + (tyy + l3) * (myy / mm) + (tzz + l5) * (mzz / mm) +
             T(2) * ((txy + l1) * (mxy / mm) + (txz + l2) * (mxz / mm) + (tyz + l4) * (myz / mm));
      } else {
        const T s = T(I.dyn_d2h + I.les_d2) * nh;
        const T mxx = s * hxx - f[8], mxy = s * hxy - f[9], mxz = s * hxz - f[10];
        const T myy = s * hyy - f[11], myz = s * hyz - f[12], mzz = -mxx - myy;
        const T lm = l0 * mxx + l3 * myy + l5 * mzz + T(2) * (l1 * mxy + l2 * mxz + l4 * myz);
        const T mm = mxx * mxx + myy * myy + mzz * mzz + T(2) * (mxy * mxy + mxz * mxz + myz * myz);
        cv = T(0.5) * (lm / mm);
      }
      // max(-1, min(1, c)) with Julia's NaN propagation
      if (!isnan(cv)) cv = cv > T(1) ? T(1) : (cv < T(-1) ? T(-1) : cv);
      o[0] = cv;
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
  const int slot0 = STAGE == 0 ? 0 : DYN_SLOT_C;
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
