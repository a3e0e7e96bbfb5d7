// Band-basis stages: U^dagger X U rotation (stage 3) and the fused Berry-curvature /
// Fermi-level scan (stage 4) for the AHC calculator.
//
// rotate:      data_K/data_K.py:130-132 (_rotate) and data_K/data_K_R.py:69-97 (Xbar,
//              with the 1/2 (X + X^dagger) symmetrisation of fourier/fft.py:183-186 applied
//              after the rotation -- U^dagger (X+X^dagger) U / 2 = (Y + Y^dagger) / 2).
// berry_omega: formula/covariant.py:161-203 (Omega) traced over the band groups of
//              data_K/data_K.py:172-198 + grid/tetrahedron.py:132-162 and binned like
//              calculators/static.py:103-136 (histogram at ceil((E - EFmin)/dEF); the
//              cumulative sum over Fermi levels is taken by scan_finalize).
#include <float.h>
#include "wbgpu_common.cuh"
#include "wbgpu_df64.cuh"
#include "wbgpu_fixed.cuh"
#include "wbgpu_band.cuh"
#include "wbgpu_tune.cuh"
#include "wbgpu_spin.cuh"

namespace {

// Real helpers of the rotation kernels in each arithmetic (float, double, double-float).
template <typename T> WBG_D T rzero() { return T(0); }
template <> WBG_D df64 rzero<df64>() { return df_from_f(0.0f); }
template <typename T> WBG_D T rhalf(T x) { return x * T(0.5); }
template <> WBG_D df64 rhalf<df64>(df64 x) { x.hi *= 0.5f; x.lo *= 0.5f; return x; }  // exact
template <typename T> WBG_D T rnan() { return T(0) / T(0); }
template <> WBG_D df64 rnan<df64>() {
  const float q = __int_as_float(0x7fffffff);
  df64 r;
  r.hi = q;
  r.lo = q;
  return r;
}
// Stored rotation output: the arithmetic's own complex type, or complex64 rounded once from a
// double-float result (the mixed path above nw = 32)
template <typename VO, typename V> WBG_D VO rstore(V a) { return a; }
template <> WBG_D float2 rstore<float2, cdf>(cdf a) { return make_float2(a.x.hi + a.x.lo, a.y.hi + a.y.lo); }
template <typename V> WBG_D V real_only(V a) { a.y = a.y - a.y; return a; }
template <> WBG_D cdf real_only<cdf>(cdf a) { a.y = df_from_f(0.0f); return a; }
// (a + conj(b)) / 2: the (m, n) element of the Hermitian part from Y_mn = a and Y_nm = b
template <typename V> WBG_D V herm_pair(V a, V b) {
  V r;
  r.x = rhalf(a.x + b.x);
  r.y = rhalf(a.y - b.y);
  return r;
}

// Element i = m*nw + n of input field src.  lower: src holds only its lower triangle (m >= n)
// of a Hermitian matrix; the upper triangle is the conjugate mirror, the diagonal is real.
template <typename V>
WBG_D V load_field(const V* src, int i, int nw, bool lower) {
  if (!lower) return src[i];
  const int m = i / nw, n = i % nw;
  V v = src[m >= n ? i : n * nw + m];
  if (m < n) v.y = -v.y;
  if (m == n) v = real_only(v);
  return v;
}

// ---------------------------------------------------------------------------------------
// rotation: Xbar[k][f] = U^dagger X[k][fsel[f]] U  (optionally Hermitian-symmetrised)
// herm[f] bits 0-1: 0 plain, 1 Hermitian part, 2 diagonal (real) only; bit 2: X[fsel[f]]
// holds only its lower triangle (wbg_r2k_columns output).
// grid: nk blocks of 256 threads; shared: U, X, T (nw*nw each, precision T)
// ---------------------------------------------------------------------------------------
template <typename T, typename VO>
__global__ void rotate_kernel(const typename C2<T>::t* __restrict__ U, long long strideU, const typename C2<T>::t* __restrict__ X,
                              int nFin, const int* __restrict__ fsel, const int* __restrict__ herm, int nFrot,
                              VO* __restrict__ Xbar, int nw) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smr[];
  V* Us = reinterpret_cast<V*>(smr);
  V* Xs = Us + nw * nw;
  V* Ts = Xs + nw * nw;
  const long long k = blockIdx.x;
  const int nw2 = nw * nw;
  for (int i = threadIdx.x; i < nw2; i += blockDim.x) Us[i] = U[k * strideU + i];
  for (int f = 0; f < nFrot; ++f) {
    const int fs = fsel[f];
    const bool fok = fs >= 0 && fs < nFin;  // selection lives in device memory: validate here
    const V* src = X + (k * nFin + (fok ? fs : 0)) * (long long)nw2;
    const T nan = rnan<T>();
    const bool lower = (herm[f] & 4) != 0;
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) Xs[i] = fok ? load_field(src, i, nw, lower) : mkc<T>(nan, nan);
    __syncthreads();
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) {  // T = X U
      const int m = i / nw, n = i % nw;
      V acc = czero<V>();
      for (int j = 0; j < nw; ++j) cfma(acc, Xs[m * nw + j], Us[j * nw + n]);
      Ts[i] = acc;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) {  // Y = U^dagger T
      const int m = i / nw, n = i % nw;
      V acc = czero<V>();
      for (int j = 0; j < nw; ++j) cfmac(acc, Us[j * nw + m], Ts[j * nw + n]);
      Xs[i] = acc;
    }
    __syncthreads();
    VO* dst = Xbar + (k * nFrot + f) * (long long)nw2;
    const bool h = (herm[f] & 3) != 0;
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) {
      V y = Xs[i];
      if (h) {
        const int m = i / nw, n = i % nw;
        y = herm_pair(y, Xs[n * nw + m]);
      }
      dst[i] = rstore<VO>(y);
    }
    __syncthreads();
  }
}

// Register-tiled rotation for nw % 4 == 0: each thread owns a 4x4 tile of the nw x nw
// output; KB k-points per CTA.  X rows are padded (stride nw+1) so the column reads of
// different tile rows fall in different banks.  Same math as rotate_kernel.
template <typename T, typename VO>
__global__ void rotate_tiled(const typename C2<T>::t* __restrict__ U, long long strideU,
                             const typename C2<T>::t* __restrict__ X, int nFin, const int* __restrict__ fsel,
                             const int* __restrict__ herm, int nFrot, VO* __restrict__ Xbar, int nw,
                             int nk, int KB) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smr[];
  const int nt = nw / 4;                 // tiles per dimension
  const int tpk = nt * nt;               // threads per k-point
  const int kl = threadIdx.x / tpk, tid = threadIdx.x % tpk;
  const int ty = tid / nt, tx = tid % nt;
  const int ldx = nw + 1;
  V* base = reinterpret_cast<V*>(smr) + (size_t)kl * (nw * nw + nw * ldx + nw * nw);
  V* Us = base;                          // [nw][nw]
  V* Xs = Us + nw * nw;                  // [nw][nw+1]
  V* Ts = Xs + nw * ldx;                 // [nw][nw]
  long long k = (long long)blockIdx.x * KB + kl;
  const bool valid = k < nk;
  if (!valid) k = nk - 1;
  const int nw2 = nw * nw;
  for (int i = tid; i < nw2; i += tpk) Us[i] = U[k * strideU + i];
  const int m0 = 4 * ty, n0 = 4 * tx;
  for (int f = 0; f < nFrot; ++f) {
    const int fs = fsel[f];
    const bool fok = fs >= 0 && fs < nFin;  // selection lives in device memory: validate here
    const V* src = X + (k * nFin + (fok ? fs : 0)) * (long long)nw2;
    const T nan = rnan<T>();
    const bool lower = (herm[f] & 4) != 0;
    for (int i = tid; i < nw2; i += tpk)
      Xs[(i / nw) * ldx + (i % nw)] = fok ? load_field(src, i, nw, lower) : mkc<T>(nan, nan);
    __syncthreads();
    V acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = czero<V>();
    for (int j = 0; j < nw; ++j) {  // T = X U
      V xa[4], ub[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) xa[a] = Xs[(m0 + a) * ldx + j];
#pragma unroll
      for (int b = 0; b < 4; ++b) ub[b] = Us[j * nw + n0 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) cfma(acc[a][b], xa[a], ub[b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) Ts[(m0 + a) * nw + n0 + b] = acc[a][b];
    __syncthreads();
    const int hmode = herm[f] & 3;
    if (hmode == 2) {  // diagonal only: Y_mm = sum_j conj(U_jm) T_jm, Hermitian part = Re
      VO* dstd = Xbar + (k * nFrot + f) * (long long)nw2;
      for (int m = tid; m < nw; m += tpk) {
        V y = czero<V>();
        for (int j = 0; j < nw; ++j) cfmac(y, Us[j * nw + m], Ts[j * nw + m]);
        if (valid) dstd[m * nw + m] = rstore<VO>(real_only(y));
      }
      __syncthreads();
      continue;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = czero<V>();
    for (int j = 0; j < nw; ++j) {  // Y = U^dagger T
      V ua[4], tb[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) ua[a] = Us[j * nw + m0 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) tb[b] = Ts[j * nw + n0 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) cfmac(acc[a][b], ua[a], tb[b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) Xs[(m0 + a) * ldx + n0 + b] = acc[a][b];
    __syncthreads();
    VO* dst = Xbar + (k * nFrot + f) * (long long)nw2;
    const bool h = hmode != 0;
    if (valid) {
      for (int i = tid; i < nw2; i += tpk) {
        const int m = i / nw, n = i % nw;
        V y = Xs[m * ldx + n];
        if (h) y = herm_pair(y, Xs[n * ldx + m]);
        dst[i] = rstore<VO>(y);
      }
    }
    __syncthreads();
  }
}

WBG_D int group_sum_i(int v, int L) {
  for (int off = L / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
WBG_D double group_sum_d(double v, int L) {
  for (int off = L / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
WBG_D int group_min_i(int v, int L) {
  for (int off = L / 2; off > 0; off >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

template <typename T> WBG_D T recip_gap(double dE);
template <> WBG_D double recip_gap<double>(double dE) { return 1.0 / dE; }
// FP64 difference (no cancellation loss), FP32 reciprocal
template <> WBG_D float recip_gap<float>(double dE) { return 1.0f / (float)dE; }
// FP64 difference, double-float reciprocal
template <> WBG_D df64 recip_gap<df64>(double dE) { return df_from_f(1.0f) / df_from(dE); }

// a stored complex element in the arithmetic's complex type (FP32 storage, double-float arithmetic)
template <typename V, typename S> WBG_D V ld_c(S a) { return a; }
template <> WBG_D cdf ld_c<cdf, float2>(float2 a) {
  cdf r;
  r.x = df_from_f(a.x);
  r.y = df_from_f(a.y);
  return r;
}
// acc += a b and acc -= a b of the complex accumulators: plain FMAs for float / double; for
// double-float lazily (df_lazy_fma: the error terms gathered in lo, renormalised once by cdone)
template <typename V> WBG_D void cmac(V& acc, const V& a, const V& b) { cfma(acc, a, b); }
template <typename V> WBG_D void cmsub(V& acc, const V& a, const V& b) { acc = csub(acc, cmul(a, b)); }
template <typename V> WBG_D V cdone(V a) { return a; }
template <> WBG_D void cmac<cdf>(cdf& acc, const cdf& a, const cdf& b) {
  df_lazy_fma(acc.x, a.x, b.x);
  df_lazy_fma(acc.x, -a.y, b.y);
  df_lazy_fma(acc.y, a.x, b.y);
  df_lazy_fma(acc.y, a.y, b.x);
}
template <> WBG_D void cmsub<cdf>(cdf& acc, const cdf& a, const cdf& b) {
  df_lazy_fma(acc.x, -a.x, b.x);
  df_lazy_fma(acc.x, a.y, b.y);
  df_lazy_fma(acc.y, -a.x, b.y);
  df_lazy_fma(acc.y, -a.y, b.x);
}
template <> WBG_D cdf cdone<cdf>(cdf a) {
  a.x = df_lazy_done(a.x);
  a.y = df_lazy_done(a.y);
  return a;
}
WBG_D double to_dbl(float x) { return (double)x; }
WBG_D double to_dbl(double x) { return x; }
WBG_D double to_dbl(df64 x) { return df_to_double(x); }

// 1/(E_n - E_l), 0 below 1e-7 (degenerate pairs).  FP64 path: native doubles.  FP32 path: the
// energies are held as double-float pairs (Eh + El = E to 48 bits); Eh_n - Eh_l is exact when
// the two are within a factor of two, so the gap keeps FP32 relative accuracy however close
// the bands, and nothing runs on the FP64 pipe.
template <typename T> WBG_D T inv_gap(const double* E, const float* Eh, const float* El, int n, int l);
template <> WBG_D double inv_gap<double>(const double* E, const float*, const float*, int n, int l) {
  const double dE = E[n] - E[l];
  return fabs(dE) < 1e-7 ? 0.0 : 1.0 / dE;
}
template <> WBG_D float inv_gap<float>(const double*, const float* Eh, const float* El, int n, int l) {
  const float dE = (Eh[n] - Eh[l]) + (El[n] - El[l]);
  return fabsf(dE) < 1e-7f ? 0.0f : __frcp_rn(dE);
}

// Trace accumulator: a double in the FP64 path; in the FP32 path a float sum with its
// rounding error carried along (Knuth two-sum), ~2^-48 relative, all on the FP32 pipe.
template <typename T> struct TraceSum;
template <> struct TraceSum<double> {
  double s = 0.0;
  WBG_D void add(double x) { s += x; }
  WBG_D double value() const { return s; }
};
template <> struct TraceSum<float> {
  float s = 0.0f, c = 0.0f;
  WBG_D void add(float x) {
    const float t = s + x;
    const float v = t - s;
    c += (s - (t - v)) + (x - v);
    s = t;
  }
  WBG_D double value() const { return (double)s + (double)c; }
};

// ---------------------------------------------------------------------------------------
// Row-panel rotation for large nw (the per-k matrices do not fit in shared memory together).
// CTA = (row panel p of RP rows, field f, k-point): W = U[:, panel]^dagger Xh  (RP x nw), then
// Y[panel, :] = W U, with Xh and U streamed through shared memory in chunks of KC rows.
// Hermitian-part fields (herm 1, 2) are symmetrised on input, Xh = (X + X^dagger)/2 -- the
// same Hermitian part (U^dagger X U + its adjoint)/2 -- and lower-triangle inputs (bit 2)
// are mirrored; herm 2 writes the real diagonal only.  Threads own 4 x 4 output tiles.
// ---------------------------------------------------------------------------------------
constexpr int PANEL_RP = 32, PANEL_KC = 16;

template <typename V>
WBG_D V herm_in(const V* src, int i, int j, int nw, int mode) {  // element (i, j) of the rotated input
  if (mode == 2) return load_field(src, i * nw + j, nw, true);     // lower triangle, mirrored
  if (mode == 1) return herm_pair(src[i * nw + j], src[j * nw + i]);  // Hermitian part
  return src[i * nw + j];
}

template <typename T, typename VO>
__global__ void __launch_bounds__(256) rotate_panel(const typename C2<T>::t* __restrict__ U, long long strideU,
                                                    const typename C2<T>::t* __restrict__ X, int nFin,
                                                    const int* __restrict__ fsel, const int* __restrict__ herm,
                                                    int nFrot, VO* __restrict__ Xbar, int nw, int nk) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smp[];
  const int np = (nw + PANEL_RP - 1) / PANEL_RP;
  const long long b = blockIdx.x;
  const int p = (int)(b % np), f = (int)((b / np) % nFrot);
  const long long k = b / ((long long)np * nFrot);
  if (k >= nk) return;
  const int r0 = p * PANEL_RP;
  const int ldw = nw + 1;
  V* Ws = reinterpret_cast<V*>(smp);        // [RP][nw+1]
  V* Cs = Ws + PANEL_RP * ldw;               // [KC][nw] chunk of Xh (phase 1) or U (phase 2)
  V* Us = Cs + PANEL_KC * nw;                // [KC][RP] chunk of U[:, panel]
  const int tx = threadIdx.x % ((nw + 3) / 4), ty = threadIdx.x / ((nw + 3) / 4);  // ty < RP/4
  const int fs = fsel[f];
  const bool fok = fs >= 0 && fs < nFin;  // selection lives in device memory: validate here
  const int hm = herm[f];
  const int inmode = (hm & 4) ? 2 : ((hm & 3) != 0 ? 1 : 0);
  const V* src = X + (k * nFin + (fok ? fs : 0)) * (long long)nw * nw;
  const V* Uk = U + k * strideU;
  const T nan = rnan<T>();
  V acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = czero<V>();
  // phase 1: W[a][j] = sum_i conj(U[i][r0 + a]) Xh[i][j]
  for (int i0 = 0; i0 < nw; i0 += PANEL_KC) {
    for (int e = threadIdx.x; e < PANEL_KC * nw; e += blockDim.x) {
      const int ii = e / nw, j = e % nw, i = i0 + ii;
      Cs[e] = i < nw ? (fok ? herm_in(src, i, j, nw, inmode) : mkc<T>(nan, nan)) : czero<V>();
    }
    for (int e = threadIdx.x; e < PANEL_KC * PANEL_RP; e += blockDim.x) {
      const int ii = e / PANEL_RP, a = e % PANEL_RP, i = i0 + ii;
      Us[e] = (i < nw && r0 + a < nw) ? Uk[i * nw + r0 + a] : czero<V>();
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < PANEL_KC; ++ii) {
      V ua[4], xb[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) ua[a] = Us[ii * PANEL_RP + 4 * ty + a];
#pragma unroll
      for (int c = 0; c < 4; ++c) xb[c] = (4 * tx + c < nw) ? Cs[ii * nw + 4 * tx + c] : czero<V>();
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) cfmac(acc[a][c], ua[a], xb[c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (4 * tx + c < nw) Ws[(4 * ty + a) * ldw + 4 * tx + c] = acc[a][c];
      acc[a][c] = czero<V>();
    }
  __syncthreads();
  // phase 2: Y[r0 + a][n] = sum_j W[a][j] U[j][n]
  for (int j0 = 0; j0 < nw; j0 += PANEL_KC) {
    for (int e = threadIdx.x; e < PANEL_KC * nw; e += blockDim.x) {
      const int jj = e / nw, n = e % nw, j = j0 + jj;
      Cs[e] = j < nw ? Uk[j * nw + n] : czero<V>();
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < PANEL_KC; ++jj) {
      if (j0 + jj >= nw) break;
      V wa[4], ub[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) wa[a] = Ws[(4 * ty + a) * ldw + j0 + jj];
#pragma unroll
      for (int c = 0; c < 4; ++c) ub[c] = (4 * tx + c < nw) ? Cs[jj * nw + 4 * tx + c] : czero<V>();
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) cfma(acc[a][c], wa[a], ub[c]);
    }
    __syncthreads();
  }
  VO* dst = Xbar + (k * nFrot + f) * (long long)nw * nw;
  // Hermitian part (herm 1): the lower triangle computed by this panel is written together
  // with its conjugate mirror and the diagonal is taken real, so the stored matrix is Hermitian
  // bit for bit (the consumers' pair terms rely on X_ln = conj(X_nl) exactly); the panel's
  // upper-triangle products are dropped -- the panel of their row writes them.
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int m = r0 + 4 * ty + a, n = 4 * tx + c;
      if (m >= nw || n >= nw) continue;
      if ((hm & 3) == 2) {
        if (m == n) dst[m * nw + n] = rstore<VO>(real_only(acc[a][c]));
      } else if ((hm & 3) == 1) {
        if (m == n) {
          dst[m * nw + n] = rstore<VO>(real_only(acc[a][c]));
        } else if (m > n) {
          dst[m * nw + n] = rstore<VO>(acc[a][c]);
          dst[n * nw + m] = rstore<VO>(cconj(acc[a][c]));
        }
      } else {
        dst[m * nw + n] = rstore<VO>(acc[a][c]);
      }
    }
}

// ---------------------------------------------------------------------------------------
// Per-band values for the tetrahedron method (wbg_band_values).  sel[k][n]: 2 = band n is in
// the Fermi-sea group [0, bandmax) (a prefix of the bands), 1 = its degenerate group is in the
// Fermi window, 0 = not needed.  With sel set, a formula kernel takes its groups from sel
// instead of the energy window and writes P[k][n][c] in place of the histogram: the group
// trace divided by the group size for sel 1, the whole sea-group trace on band 0 for sel 2,
// zero otherwise -- so that sum_n P[k][n] w_n(E_F) with per-band tetrahedron weights w_n is
// the reference's sum over groups of trace x group-averaged weight.
// ---------------------------------------------------------------------------------------
struct BandSel {
  const signed char* sel;
  double* P;
};

WBG_D int sel_bandmax(const signed char* selk, int nw, int lane, int L) {
  int c = 0;
  for (int n = lane; n < nw; n += L) c += selk[n] == 2;
  return group_sum_i(c, L);
}

// additive formulas: t[n * ts + c] is band n's row of the trace of its group (or of the sea)
WBG_D void emit_band_values(double* P, long long k, int nw, int nc, int lane, int L, int bandmax,
                            const signed char* selk, const int* myS, const double* t, int ts) {
  for (int n = lane; n < nw; n += L) {
    int qs = 0, qe = 0;  // bands summed into band n's value, times scale
    double scale = 1.0;
    if (n < bandmax) {
      if (n == 0) qe = bandmax;
    } else if (selk[n] == 1) {
      qs = n;
      qe = n + 1;
      while (!myS[qs]) --qs;
      while (qe < nw && !myS[qe]) ++qe;
      scale = 1.0 / (double)(qe - qs);
    }
    for (int c = 0; c < nc; ++c) {
      double v = 0.0;
      for (int q = qs; q < qe; ++q) v += t[q * ts + c];
      P[(k * nw + n) * nc + c] = v * scale;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Fused Omega traces + Fermi-level histogram.
// grid: persistent blocks of G*L threads; each group of L lanes takes one k-point at a time.
// Xbar layout: [k][nFbar][nw][nw]; V at iV..iV+2, A at iA..iA+2, O(rotAA) at iO..iO+2.
// hist: [nEF][3] doubles, accumulated with atomics (FP64).
// ---------------------------------------------------------------------------------------
// With tab != nullptr (tabulation, calculators/tabulate.py:21-52): no histogram; every band n
// gets the average over its degenerate group of the trace, the energy and Re V_nn, written to
// tab[k][n][0..6] = (E, V_x, V_y, V_z, Omega_x, Omega_y, Omega_z).  The caller passes an
// unbounded window (EFmin = -inf, EFmax = +inf), so there is no sea group.
template <typename T>
__global__ void berry_omega_kernel(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar,
                                   int iV, int iA, int iO, int nw, int nk, int L, int G, WbgScan sp, int internal_terms,
                                   int external_terms, wbg_u64* __restrict__ hist, int shist, double* __restrict__ tab,
                                   BandSel bs) {
  typedef typename C2<T>::t V;
  extern __shared__ double smb[];
  const int nh = 3 * sp.nEF;  // histogram entries [nEF][3]
  // the block's histogram in shared memory (order-independent fixed point), or, when it does not
  // fit, the global one directly
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);      // [G][nw]
  double* tv = Es + G * nw;                           // [G][nw][3]
  float* Ehl = reinterpret_cast<float*>(tv + 3 * G * nw);  // [G][2][nw]: double-float energies
  int* start = reinterpret_cast<int*>(Ehl + 2 * G * nw);   // [G][nw]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = tv + 3 * grp * nw;
  float* myEh = Ehl + 2 * grp * nw;
  float* myEl = myEh + nw;
  int* myS = start + grp * nw;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
    for (int i = lane; i < nw; i += L) {
      const double e = E[kk * nw + i];
      const float eh = (float)e;
      myE[i] = e;
      myEh[i] = eh;
      myEl[i] = (float)(e - (double)eh);
    }
    __syncwarp();
    for (int i = lane; i < nw; i += L) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    __syncwarp();
    int bandmax;
    if (bs.sel) {
      bandmax = sel_bandmax(bs.sel + kk * nw, nw, lane, L);
    } else {
      int below = 0, f0 = nw;
      for (int n = lane; n < nw; n += L) {
        below += myE[n] < sp.EFmin;
        if (myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) f0 = min(f0, n);
        }
      }
      below = group_sum_i(below, L);
      f0 = group_min_i(f0, L);
      bandmax = min(below, f0);
    }
    const V* Xk = Xbar + kk * nFbar * nw2;
    for (int n = lane; n < nw; n += L) {
      int gs = n, ge = n + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      bool ingroup;
      if (n < bandmax) { gs = 0; ge = bandmax; ingroup = true; }
      else ingroup = bs.sel ? bs.sel[kk * nw + n] == 1 : (myE[ge - 1] >= sp.EFmin && myE[gs] <= sp.EFmax);
      double t[3] = {0.0, 0.0, 0.0};
      if (ingroup) {
        TraceSum<T> sr[3];  // real part of the trace; its imaginary part is not needed
        for (int l = 0; l < nw; ++l) {
          if (l >= gs && l < ge) continue;
          const T dinv = inv_gap<T>(myE, myEh, myEl, n, l);
          V Dnl[3], Dln[3], Aln[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            Dnl[a] = cscale(Xk[(iV + a) * nw2 + n * nw + l], -dinv);  // D_nl = -V_nl / (E_n - E_l)
            Dln[a] = cscale(Xk[(iV + a) * nw2 + l * nw + n], dinv);   // D_ln = -V_ln / (E_l - E_n)
            Aln[a] = external_terms ? Xk[(iA + a) * nw2 + l * nw + n] : czero<V>();
          }
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            V acc = czero<V>();
            if (internal_terms) acc = cmuli(cmul(Dnl[al], Dln[be]));  // i D D (sign applied below)
            V accx = czero<V>();
            if (external_terms) { cfma(accx, Dnl[be], Aln[al]); accx = csub(accx, cmul(Dnl[al], Aln[be])); }
            // Re S += Re[-i D^a_nl D^b_ln - D^a_nl A^b_ln + D^b_nl A^a_ln]
            sr[g].add(accx.x - acc.x);
          }
        }
        if (external_terms) {
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            sr[g].add((T)0.5 * Xk[(iO + g) * nw2 + n * nw + n].x);
            V acc = czero<V>();
            for (int np = gs; np < ge; ++np) cfma(acc, Xk[(iA + al) * nw2 + n * nw + np], Xk[(iA + be) * nw2 + np * nw + n]);
            sr[g].add(acc.y);  // Re(-i acc)
          }
        }
        for (int g = 0; g < 3; ++g) t[g] = 2.0 * sr[g].value();
      }
      for (int g = 0; g < 3; ++g) myT[n * 3 + g] = t[g];
    }
    __syncwarp();
    if (valid && tab) {
      for (int n = lane; n < nw; n += L) {
        int gs = n, ge = n + 1;
        while (!myS[gs]) --gs;
        while (ge < nw && !myS[ge]) ++ge;
        double v[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int q = gs; q < ge; ++q) {
          v[0] += myE[q];
          for (int a = 0; a < 3; ++a) v[1 + a] += (double)Xk[(iV + a) * nw2 + q * nw + q].x;
          for (int g = 0; g < 3; ++g) v[4 + g] += myT[q * 3 + g];
        }
        const double inv = 1.0 / (double)(ge - gs);
        for (int i = 0; i < 7; ++i) tab[(k * nw + n) * 7 + i] = v[i] * inv;
      }
    } else if (valid && bs.P) {
      emit_band_values(bs.P, k, nw, 3, lane, L, bandmax, bs.sel + k * nw, myS, myT, 3);
    } else if (valid) {
      for (int n = lane; n < nw; n += L) {
        int gs = -1, ge = -1;
        bool sea = false;
        if (n == 0 && bandmax > 0) { gs = 0; ge = bandmax; sea = true; }
        else if (n >= bandmax && myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { gs = n; ge = g1; }
        }
        if (gs < 0) continue;
        double v[3] = {0.0, 0.0, 0.0}, esum = 0.0;
        for (int q = gs; q < ge; ++q) {
          for (int g = 0; g < 3; ++g) v[g] += myT[q * 3 + g];
          esum += myE[q];
        }
        int bin = -1;
        if (sea) bin = 0;
        else {
          const double Em = esum / (double)(ge - gs);
          if (Em < sp.EFmin) bin = 0;
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int g = 0; g < 3; ++g) fx_add_double(sh + 2 * (bin * 3 + g), v[g], sh + 2 * nh);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (hist && shist) fx_flush(sh, nh, hist);
}

// ---------------------------------------------------------------------------------------
// Omega traces for exactly Hermitian V and A in FP32 (the mixed path: lower-triangle inputs,
// Hermitian rotation outputs), nw <= 32 C.  Lane l owns the bands (columns) l + 32 j, j < C,
// and the warp walks the rows n, so every load is a coalesced row segment.  Each band sums its
// own trace.  For a pair (l, n) in different degenerate groups the term of band l is
// T(l, n) = Re[-i D^a_ln D^b_nl - D^a_ln A^b_nl + D^b_ln A^a_nl] = -T(n, l) (D anti-Hermitian,
// A Hermitian); the two lanes that meet the pair both evaluate the one canonical term T(p, q),
// p = min(l, n), q = max(l, n), from the element X_pq (X_nl itself, or the conjugate of it,
// which is X_ln bit for bit), with the same arithmetic, so the two bands receive +T and -T
// exactly.  Over any set of bands the scan adds together (the Fermi sea, or every level above
// two groups) the pair terms then cancel without FP32 residue -- the terms of near-degenerate
// pairs, |V|^2 / dE^2, can be 10^4 times the result.  A band's sum is compensated (TraceSum)
// and kept as a double.  The sea group's trace is the sum of its bands' traces over their own
// degenerate groups: equal to the reference's sea trace in exact arithmetic, since the
// cross-group A A terms inside the sea cancel pairwise as well.  Grouping and binning as in
// berry_omega_kernel.  One warp per k-point, G warps per block.
// ---------------------------------------------------------------------------------------
template <int C>
__global__ void berry_omega_cols(const double* __restrict__ E, const float2* __restrict__ Xbar, int nFbar, int iV,
                                 int iA, int iO, int nw, int nk, int G, WbgScan sp, int internal_terms,
                                 int external_terms, wbg_u64* __restrict__ hist, int shist) {
  constexpr int NWM = 32 * C;
  extern __shared__ double smb[];
  const int nh = 3 * sp.nEF;  // histogram entries [nEF][3], fixed point (shared or global)
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);            // [G][NWM]
  double* tv = Es + G * NWM;                                // [G][NWM][3]
  float* Ehl = reinterpret_cast<float*>(tv + 3 * G * NWM);  // [G][2][NWM]
  int* start = reinterpret_cast<int*>(Ehl + 2 * G * NWM);   // [G][NWM]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* myE = Es + grp * NWM;
  double* myT = tv + 3 * grp * NWM;
  float* myEh = Ehl + 2 * grp * NWM;
  float* myEl = myEh + NWM;
  int* myS = start + grp * NWM;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const int i = lane + 32 * j;
      if (i < nw) {
        const double e = E[kk * nw + i];
        const float eh = (float)e;
        myE[i] = e;
        myEh[i] = eh;
        myEl[i] = (float)(e - (double)eh);
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const int i = lane + 32 * j;
      if (i < nw) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    }
    __syncwarp();
    int below = 0, f0 = nw;
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const int i = lane + 32 * j;
      if (i < nw) {
        below += myE[i] < sp.EFmin;
        if (myS[i]) {
          int g1 = i + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[i] <= sp.EFmax) f0 = min(f0, i);
        }
      }
    }
    below = group_sum_i(below, 32);
    f0 = group_min_i(f0, 32);
    const int bandmax = min(below, f0);
    // own bands: degenerate group [gs, ge) and whether the scan reads the band
    int gs[C], ge[C];
    bool need[C];
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const int l = lane + 32 * j;
      gs[j] = ge[j] = 0;
      need[j] = false;
      if (l < nw) {
        int a = l, b = l + 1;
        while (!myS[a]) --a;
        while (b < nw && !myS[b]) ++b;
        gs[j] = a;
        ge[j] = b;
        need[j] = l < bandmax || (myE[b - 1] >= sp.EFmin && myE[a] <= sp.EFmax);
      }
    }
    TraceSum<float> acc[C][3];
    const float2* Xk = Xbar + kk * nFbar * nw2;
    for (int n = 0; n < nw; ++n) {  // warp-uniform
#pragma unroll
      for (int j = 0; j < C; ++j) {
        const int l = lane + 32 * j;
        if (l >= nw || !need[j]) continue;
        float2 Vn[3], An[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          Vn[a] = Xk[(iV + a) * nw2 + n * nw + l];
          An[a] = external_terms ? Xk[(iA + a) * nw2 + n * nw + l] : make_float2(0.f, 0.f);
        }
        if (n < gs[j] || n >= ge[j]) {
          // canonical pair (p, q) = (min, max): X_pq = X_nl if n < l, else X_ln = conj(X_nl)
          const bool np = n < l;
          const int p = np ? n : l, q = np ? l : n;
          const float dinv = inv_gap<float>(myE, myEh, myEl, p, q);  // 1 / (E_p - E_q)
          float2 Dpq[3], Dqp[3], Aqp[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float2 vpq = np ? Vn[a] : cconj(Vn[a]);
            const float2 apq = np ? An[a] : cconj(An[a]);
            Dpq[a] = cscale(vpq, -dinv);        // D_pq = -V_pq / (E_p - E_q)
            Dqp[a] = cscale(cconj(vpq), dinv);  // D_qp = -V_qp / (E_q - E_p), V_qp = conj(V_pq)
            Aqp[a] = cconj(apq);                // A_qp = conj(A_pq)
          }
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            float2 dd = czero<float2>(), dx = czero<float2>();
            if (internal_terms) dd = cmuli(cmul(Dpq[al], Dqp[be]));
            if (external_terms) { cfma(dx, Dpq[be], Aqp[al]); dx = csub(dx, cmul(Dpq[al], Aqp[be])); }
            const float t = dx.x - dd.x;  // T(p, q) = Re[-i D^a_pq D^b_qp - D^a_pq A^b_qp + D^b_pq A^a_qp]
            acc[j][g].add(np ? -t : t);   // band l = q receives T(q, p) = -T(p, q)
          }
        } else if (external_terms) {  // n in l's group: Re(-i A^a_ln A^b_nl), plus 1/2 O_ll
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            acc[j][g].add(cmul(cconj(An[al]), An[be]).y);
            if (l == n) acc[j][g].add(0.5f * Xk[(iO + g) * nw2 + n * nw + n].x);
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < C; ++j) {
      const int l = lane + 32 * j;
      if (l < nw)
        for (int g = 0; g < 3; ++g) myT[l * 3 + g] = need[j] ? 2.0 * acc[j][g].value() : 0.0;
    }
    __syncwarp();
    if (valid) {
#pragma unroll
      for (int j = 0; j < C; ++j) {
        const int n = lane + 32 * j;
        if (n >= nw) continue;
        int g0 = -1, g1 = -1;
        bool sea = false;
        if (n == 0 && bandmax > 0) { g0 = 0; g1 = bandmax; sea = true; }
        else if (n >= bandmax && myS[n]) {
          int e1 = n + 1;
          while (e1 < nw && !myS[e1]) ++e1;
          if (myE[e1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { g0 = n; g1 = e1; }
        }
        if (g0 < 0) continue;
        double v[3] = {0.0, 0.0, 0.0}, esum = 0.0;
        for (int q = g0; q < g1; ++q) {
          for (int g = 0; g < 3; ++g) v[g] += myT[q * 3 + g];
          esum += myE[q];
        }
        int bin = -1;
        if (sea) bin = 0;
        else {
          const double Em = esum / (double)(g1 - g0);
          if (Em < sp.EFmin) bin = 0;
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int g = 0; g < 3; ++g) fx_add_double(sh + 2 * (bin * 3 + g), v[g], sh + 2 * nh);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (shist) fx_flush(sh, nh, hist);
}

// ---------------------------------------------------------------------------------------
// Generic Fermi-level scan of additive group traces (calculators/static.py:60-169) for
//   WBG_FORMULA_IDENTITY  (formula/covariant.py:10-22; CumDOS / DOS)      1 component:  1
//   WBG_FORMULA_INVMASS   (formula/elementary.py:28-34; Ohmic_FermiSea)   9 components:
//        Re W^{bd}_nn + sum_{l out of the group} Re(V^d_nl V^b_ln + V^b_nl V^d_ln) / (E_n - E_l)
//        (the generalised derivative Wbar - D Vbar + Vbar D of formula/formula.py:95-118)
//   WBG_FORMULA_VELVEL    (formula/covariant.py:817-820; Ohmic_FermiSurf) 9 components:
//        sum_{n' in the group} Re V^a_nn' V^b_n'n
//   WBG_FORMULA_DIAG      (formula/covariant.py:331-335; Spin)            3 components:
//        Re X^c_nn of the 3-component field starting at iV
// per band n; the group sums are binned like the Omega kernel.  sea != 0: Fermi-sea groups
// (E below the window add to every level, the sea group); sea == 0: Fermi-surface groups only.
// hist [nEF][ncomp] (component (b, d) at 3 b + d).
// ---------------------------------------------------------------------------------------
__host__ __device__ inline int scan_ncomp(int formula) {
  return formula == WBG_FORMULA_IDENTITY ? 1
         : formula == WBG_FORMULA_DIAG   ? 3
         : (formula == WBG_FORMULA_VELVELVEL || formula == WBG_FORMULA_SPIN_OMEGA) ? 27
                                           : 9;
}

// spin Berry curvature (formula/covariant.py:759-788, SpinOmega, additive) of band n:
//   t[9 a + 3 b + s] += -2 Im( J^{as}_nl / (E_n - E_l) (D^b_ln - i Abar^b_ln) ),  l outside the group
template <typename T, int K>
__device__ void spin_omega_terms(const KBand<T>& kb, int n, int gs, int ge, double* t) {
  typedef typename C2<T>::t V;
  for (int l = 0; l < kb.nw; ++l) {
    if (l >= gs && l < ge) continue;
    V J[9], Jt[9];
    spin_current<T, K>(kb, n, l, J);
    spin_current<T, K>(kb, l, n, Jt);
    const T dnl = kb.dinv(n, l);
    V vde[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      vde[b] = kb.D(b, l, n);
      if (kb.f.external_terms) vde[b] = csub(vde[b], cmuli(kb.x(kb.f.A + b, l, n)));
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const V j = cscale(cadd(J[3 * a + s], cconj(Jt[3 * a + s])), T(0.5) * dnl);
#pragma unroll
        for (int b = 0; b < 3; ++b) t[9 * a + 3 * b + s] += -2.0 * (double)cmul(j, vde[b]).y;
      }
  }
}

// NCM: components held per band (9, or 27 for WBG_FORMULA_VELVELVEL / WBG_FORMULA_SPIN_OMEGA)
template <typename T, int NCM>
__global__ void berry_scan_kernel(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar,
                                  int iV, int iW, int nw, int nk, int L, int G, WbgScan sp, int formula, int sea,
                                  wbg_u64* __restrict__ hist, int shist, BandSel bs, wbg_dynamic_spec fs) {
  typedef typename C2<T>::t V;
  const int nc = scan_ncomp(formula);
  extern __shared__ double smb[];
  const int nh = nc * sp.nEF;  // histogram entries [nEF][nc], fixed point (shared or global)
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);      // [G][nw]
  double* tv = Es + G * nw;                           // [G][nw][NCM]
  int* start = reinterpret_cast<int*>(tv + NCM * G * nw);  // [G][nw]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = tv + NCM * grp * nw;
  int* myS = start + grp * nw;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
    for (int i = lane; i < nw; i += L) myE[i] = E[kk * nw + i];
    __syncwarp();
    for (int i = lane; i < nw; i += L) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    __syncwarp();
    int bandmax = 0;
    if (bs.sel) {
      bandmax = sel_bandmax(bs.sel + kk * nw, nw, lane, L);
    } else if (sea) {
      int below = 0, f0 = nw;
      for (int n = lane; n < nw; n += L) {
        below += myE[n] < sp.EFmin;
        if (myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) f0 = min(f0, n);
        }
      }
      below = group_sum_i(below, L);
      f0 = group_min_i(f0, L);
      bandmax = min(below, f0);
    }
    const V* Xk = Xbar ? Xbar + kk * nFbar * nw2 : nullptr;
    for (int n = lane; n < nw; n += L) {
      int gs = n, ge = n + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      if (n < bandmax) { gs = 0; ge = bandmax; }
      double t[NCM];
#pragma unroll
      for (int c = 0; c < NCM; ++c) t[c] = 0.0;
      if (formula == WBG_FORMULA_IDENTITY) {
        t[0] = 1.0;
      } else if (NCM == 27 && formula == WBG_FORMULA_VELVELVEL) {
        // sum_{n', n'' in the group} Re V^a_nn' V^b_n'n'' V^c_n''n (FormulaProduct VelVelVel)
        for (int p = gs; p < ge; ++p)
          for (int q = gs; q < ge; ++q) {
            V A3[3], B3[3], C3[3];
            for (int a = 0; a < 3; ++a) {
              A3[a] = Xk[(iV + a) * nw2 + n * nw + p];
              B3[a] = Xk[(iV + a) * nw2 + p * nw + q];
              C3[a] = Xk[(iV + a) * nw2 + q * nw + n];
            }
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) {
                const V ab = cmul(A3[a], B3[b]);
                for (int c = 0; c < 3; ++c) t[9 * a + 3 * b + c] += (double)cmul(ab, C3[c]).x;
              }
          }
      } else if (NCM == 27 && formula == WBG_FORMULA_SPIN_OMEGA) {
        KBand<T> kb;
        kb.X = Xk;
        kb.E = myE;
        kb.nw = nw;
        kb.nw2 = nw2;
        kb.f = fs;
        if (fs.formula == WBG_DYN_SHC_QIAO) spin_omega_terms<T, WBG_DYN_SHC_QIAO>(kb, n, gs, ge, t);
        else if (fs.formula == WBG_DYN_SHC_RYOO) spin_omega_terms<T, WBG_DYN_SHC_RYOO>(kb, n, gs, ge, t);
        else spin_omega_terms<T, WBG_DYN_SHC_SIMPLE>(kb, n, gs, ge, t);
      } else if (formula == WBG_FORMULA_DIAG) {
        for (int c = 0; c < 3; ++c) t[c] = (double)Xk[(iV + c) * nw2 + n * nw + n].x;
      } else if (formula == WBG_FORMULA_INVMASS) {
        for (int b = 0; b < 3; ++b)
          for (int d = 0; d < 3; ++d) t[3 * b + d] = (double)Xk[(iW + 3 * b + d) * nw2 + n * nw + n].x;
        for (int l = 0; l < nw; ++l) {
          if (l >= gs && l < ge) continue;
          const double dE = myE[n] - myE[l];
          const T dinv = fabs(dE) < 1e-7 ? T(0) : recip_gap<T>(dE);
          V Vnl[3], Vln[3];
          for (int a = 0; a < 3; ++a) {
            Vnl[a] = Xk[(iV + a) * nw2 + n * nw + l];
            Vln[a] = Xk[(iV + a) * nw2 + l * nw + n];
          }
          for (int b = 0; b < 3; ++b)
            for (int d = 0; d < 3; ++d)
              t[3 * b + d] += (double)((cmul(Vnl[d], Vln[b]).x + cmul(Vnl[b], Vln[d]).x) * dinv);
        }
      } else {  // WBG_FORMULA_VELVEL
        for (int np = gs; np < ge; ++np) {
          V Vnp[3], Vpn[3];
          for (int a = 0; a < 3; ++a) {
            Vnp[a] = Xk[(iV + a) * nw2 + n * nw + np];
            Vpn[a] = Xk[(iV + a) * nw2 + np * nw + n];
          }
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) t[3 * a + b] += (double)cmul(Vnp[a], Vpn[b]).x;
        }
      }
      for (int c = 0; c < NCM; ++c) myT[n * NCM + c] = t[c];
    }
    __syncwarp();
    if (valid && bs.P) {
      emit_band_values(bs.P, k, nw, nc, lane, L, bandmax, bs.sel + k * nw, myS, myT, NCM);
    } else if (valid) {
      for (int n = lane; n < nw; n += L) {
        int gs = -1, ge = -1;
        bool seag = false;
        if (n == 0 && bandmax > 0) { gs = 0; ge = bandmax; seag = true; }
        else if (n >= bandmax && myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { gs = n; ge = g1; }
        }
        if (gs < 0) continue;
        double v[NCM], esum = 0.0;
        for (int c = 0; c < NCM; ++c) v[c] = 0.0;
        for (int q = gs; q < ge; ++q) {
          for (int c = 0; c < nc; ++c) v[c] += myT[q * NCM + c];
          esum += myE[q];
        }
        int bin = -1;
        if (seag) bin = 0;
        else {
          const double Em = esum / (double)(ge - gs);
          if (Em < sp.EFmin) bin = 0;  // in range but below the first level: every level
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int c = 0; c < nc; ++c) fx_add_double(sh + 2 * (bin * nc + c), v[c], sh + 2 * nh);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (hist && shist) fx_flush(sh, nh, hist);
}

// ---------------------------------------------------------------------------------------
// In-group matrix products (formula/formula.py:121-151, FormulaProduct) of one to three
// factors with the factor lists of formula/covariant.py:798-865 (VelOmega, MassVel, MassMass,
// VelMassVel, VelSpin, OmegaS, OmegaOmega, VelHplus, OmegaHplus) and the single-factor DerSpin
// (formula/covariant.py:338-342).  The factors are the velocity V^a and the spin S^a (the group
// blocks of the fields), the Berry curvature Omega^c (its nn block, formula/covariant.py:161-203),
// Morb_Hpm^c with sign +1 (Morb_H + (E_p + E_q)/2 Omega, formula/covariant.py:375-449), the inverse
// mass M^{bd} (the generalised derivative of V, formula/formula.py:108-112 with
// formula/elementary.py:28-34) and the spin derivative dS^{ad} (the generalised derivative of S).
// For band n of a group G the diagonal element of the product is
//   t_n = Re F1_nn                                 (one factor)
//   t_n = Re sum_{p in G} F1_np F2_pn              (two factors)
//   t_n = Re sum_{p, q in G} F1_np F2_pq F3_qn     (three factors)
// with component (i, j[, m]) at (i d2 + j) d3 + m: the Cartesian indices of the factors one
// after another.  The group trace sum_{n in G} t_n is binned like wbg_berry_scan (with sea != 0
// the bands below the window form one group [0, bandmax)).  A factor element (p, q) with an
// l-sum runs over the bands l outside the group:
//   Omega^c_pq = s_pq + conj(s_qp),
//   s_pq = sum_l [-i D^a_pl D^b_lq - D^a_pl A^b_lq + D^b_pl A^a_lq] + O^c_pq / 2
//          - i sum_{p' in G} A^a_pp' A^b_p'q,                     (a, b) = (c + 1, c + 2) mod 3
//   M^{bd}_pq = W^{bd}_pq - sum_l D^d_pl V^b_lq + sum_l V^b_pl D^d_lq,
// D_xy = -V_xy / (E_x - E_y) (0 below 1e-7).  A lane accumulates its bands' rows t_n in
// shared memory (up to 81 components); groups of L lanes take one k-point at a time.
// ---------------------------------------------------------------------------------------
template <typename T, typename VS>
struct ProductTerms {
  typedef typename C2<T>::t V;
  const VS* X;
  const double* E;
  const float* Eh;
  const float* El;
  int nw;
  long long nw2;
  wbg_product_spec s;
  WBG_D V x(int fld, int p, int q) const {
    const VS v = X[fld * nw2 + (long long)p * nw + q];
    V r;
    r.x = (T)v.x;
    r.y = (T)v.y;
    return r;
  }
  WBG_D V D(int a, int p, int q) const { return cscale(x(s.V + a, p, q), -inv_gap<T>(E, Eh, El, p, q)); }
  // Omega^c_pq (orb = false) or Morb_H^c_pq (orb = true): s_pq + conj(s_qp) with
  //   s_pq = sum_l w_l [-i D^a_pl D^b_lq] + sum_l [-D^a_pl Y^b_lq + D^b_pl Y^a_lq] + Z^c_pq / 2
  //          - i sum_{r in G} A^a_pr w_r A^b_rq,
  // w = 1, Y = A, Z = rotA for Omega; w = E, Y = B, Z = C for Morb_H (formula/covariant.py:161-203, 375-416)
  WBG_D void curv(bool orb, int p, int q, int gs, int ge, V* out) const {
    const int fY = orb ? s.B : s.A, fZ = orb ? s.C : s.O;
    V s1[3], s2[3];  // s_pq and s_qp
#pragma unroll
    for (int c = 0; c < 3; ++c) s1[c] = s2[c] = czero<V>();
    for (int l = 0; l < nw; ++l) {
      if (l >= gs && l < ge) continue;
      const T w = orb ? (T)E[l] : T(1);
      V Dpl[3], Dlq[3], Dql[3], Dlp[3], Ylq[3], Ylp[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Dpl[a] = D(a, p, l);
        Dlq[a] = D(a, l, q);
        Dql[a] = D(a, q, l);
        Dlp[a] = D(a, l, p);
        Ylq[a] = s.external_terms ? x(fY + a, l, q) : czero<V>();
        Ylp[a] = s.external_terms ? x(fY + a, l, p) : czero<V>();
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int al = (c + 1) % 3, be = (c + 2) % 3;
        if (s.internal_terms) {
          s1[c] = csub(s1[c], cmuli(cscale(cmul(Dpl[al], Dlq[be]), w)));
          s2[c] = csub(s2[c], cmuli(cscale(cmul(Dql[al], Dlp[be]), w)));
        }
        if (s.external_terms) {
          s1[c] = cadd(s1[c], csub(cmul(Dpl[be], Ylq[al]), cmul(Dpl[al], Ylq[be])));
          s2[c] = cadd(s2[c], csub(cmul(Dql[be], Ylp[al]), cmul(Dql[al], Ylp[be])));
        }
      }
    }
    if (s.external_terms) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int al = (c + 1) % 3, be = (c + 2) % 3;
        s1[c] = cadd(s1[c], cscale(x(fZ + c, p, q), T(0.5)));
        s2[c] = cadd(s2[c], cscale(x(fZ + c, q, p), T(0.5)));
        V a1 = czero<V>(), a2 = czero<V>();
        for (int r = gs; r < ge; ++r) {
          const T w = orb ? (T)E[r] : T(1);
          cfma(a1, cscale(x(s.A + al, p, r), w), x(s.A + be, r, q));
          cfma(a2, cscale(x(s.A + al, q, r), w), x(s.A + be, r, p));
        }
        s1[c] = csub(s1[c], cmuli(a1));
        s2[c] = csub(s2[c], cmuli(a2));
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] = cadd(s1[c], cconj(s2[c]));
  }
  // generalised derivative of the 3-component field fX with its derivative fdX (9, (a, d) at
  // 3 a + d): dX^{ad}_pq - sum_l D^d_pl X^a_lq + sum_l X^a_pl D^d_lq (formula/formula.py:108-112)
  WBG_D void gender(int fX, int fdX, int p, int q, int gs, int ge, V* out) const {
#pragma unroll
    for (int i = 0; i < 9; ++i) out[i] = x(fdX + i, p, q);
    for (int l = 0; l < nw; ++l) {
      if (l >= gs && l < ge) continue;
      V Xlq[3], Xpl[3], Dpl[3], Dlq[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Xlq[a] = x(fX + a, l, q);
        Xpl[a] = x(fX + a, p, l);
        Dpl[a] = D(a, p, l);
        Dlq[a] = D(a, l, q);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) out[3 * a + d] = cadd(out[3 * a + d], csub(cmul(Xpl[a], Dlq[d]), cmul(Dpl[d], Xlq[a])));
    }
  }
  // element (p, q) of factor `kind`; returns its number of components
  WBG_D int elem(int kind, int p, int q, int gs, int ge, V* out) const {
    if (kind == WBG_FACTOR_OMEGA) { curv(false, p, q, gs, ge, out); return 3; }
    if (kind == WBG_FACTOR_MASS) { gender(s.V, s.W, p, q, gs, ge, out); return 9; }
    if (kind == WBG_FACTOR_DERSPIN) { gender(s.S, s.dS, p, q, gs, ge, out); return 9; }
    if (kind == WBG_FACTOR_HPLUS) {  // Morb_Hpm, sign +1 (formula/covariant.py:419-449)
      V om[3];
      curv(true, p, q, gs, ge, out);
      curv(false, p, q, gs, ge, om);
      const T eav = (T)(0.5 * (E[p] + E[q]));
#pragma unroll
      for (int c = 0; c < 3; ++c) out[c] = cadd(out[c], cscale(om[c], eav));
      return 3;
    }
    const int f = kind == WBG_FACTOR_SPIN ? s.S : s.V;
#pragma unroll
    for (int a = 0; a < 3; ++a) out[a] = x(f + a, p, q);
    return 3;
  }
};

// T: arithmetic (FP64 in both paths: the blocks' l-sums cancel against W and the products of up
// to three blocks amplify FP32 rounding), VS: storage of Xbar (complex64 in the mixed path)
template <typename T, typename VS>
__global__ void berry_product_kernel(const double* __restrict__ E, const VS* __restrict__ Xbar,
                                     int nFbar, wbg_product_spec ps, int nc, int nw, int nk, int L, int G, WbgScan sp,
                                     int sea, wbg_u64* __restrict__ hist, int shist, BandSel bs) {
  typedef typename C2<T>::t V;
  extern __shared__ double smb[];
  const int nh = nc * sp.nEF;
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);                  // [G][nw]
  double* tv = Es + G * nw;                                       // [G][nw][nc]
  float* Ehl = reinterpret_cast<float*>(tv + (size_t)G * nw * nc);  // [G][2][nw]
  int* start = reinterpret_cast<int*>(Ehl + 2 * G * nw);          // [G][nw]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = tv + (size_t)nc * grp * nw;
  float* myEh = Ehl + 2 * grp * nw;
  float* myEl = myEh + nw;
  int* myS = start + grp * nw;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
    for (int i = lane; i < nw; i += L) {
      const double e = E[kk * nw + i];
      const float eh = (float)e;
      myE[i] = e;
      myEh[i] = eh;
      myEl[i] = (float)(e - (double)eh);
    }
    __syncwarp();
    for (int i = lane; i < nw; i += L) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    __syncwarp();
    int bandmax = 0;
    if (bs.sel) {
      bandmax = sel_bandmax(bs.sel + kk * nw, nw, lane, L);
    } else if (sea) {
      int below = 0, f0 = nw;
      for (int n = lane; n < nw; n += L) {
        below += myE[n] < sp.EFmin;
        if (myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) f0 = min(f0, n);
        }
      }
      below = group_sum_i(below, L);
      f0 = group_min_i(f0, L);
      bandmax = min(below, f0);
    }
    ProductTerms<T, VS> pt{Xbar + kk * nFbar * nw2, myE, myEh, myEl, nw, nw2, ps};
    for (int n = lane; n < nw; n += L) {
      int gs = n, ge = n + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      bool need;
      if (n < bandmax) { gs = 0; ge = bandmax; need = true; }
      else need = bs.sel ? bs.sel[kk * nw + n] == 1 : (myE[ge - 1] >= sp.EFmin && myE[gs] <= sp.EFmax);
      double* t = myT + (size_t)n * nc;
      for (int c = 0; c < nc; ++c) t[c] = 0.0;
      if (!need) continue;
      V F1[9], F2[9], F3[9];
      if (ps.nfactors == 1) {
        const int d1 = pt.elem(ps.factor[0], n, n, gs, ge, F1);
        for (int i = 0; i < d1; ++i) t[i] += (double)F1[i].x;
      }
      for (int p = gs; p < ge && ps.nfactors > 1; ++p) {
        const int d1 = pt.elem(ps.factor[0], n, p, gs, ge, F1);
        if (ps.nfactors == 2) {
          const int d2 = pt.elem(ps.factor[1], p, n, gs, ge, F2);
          for (int i = 0; i < d1; ++i)
            for (int j = 0; j < d2; ++j) t[i * d2 + j] += (double)cmul(F1[i], F2[j]).x;
        } else {
          for (int q = gs; q < ge; ++q) {
            const int d2 = pt.elem(ps.factor[1], p, q, gs, ge, F2);
            const int d3 = pt.elem(ps.factor[2], q, n, gs, ge, F3);
            for (int i = 0; i < d1; ++i)
              for (int j = 0; j < d2; ++j) {
                const V ab = cmul(F1[i], F2[j]);
                for (int m = 0; m < d3; ++m) t[(i * d2 + j) * d3 + m] += (double)cmul(ab, F3[m]).x;
              }
          }
        }
      }
    }
    __syncwarp();
    if (valid && bs.P) {
      emit_band_values(bs.P, k, nw, nc, lane, L, bandmax, bs.sel + k * nw, myS, myT, nc);
    } else if (valid) {
      for (int n = lane; n < nw; n += L) {
        int gs = -1, ge = -1;
        bool seag = false;
        if (n == 0 && bandmax > 0) { gs = 0; ge = bandmax; seag = true; }
        else if (n >= bandmax && myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { gs = n; ge = g1; }
        }
        if (gs < 0) continue;
        double esum = 0.0;
        for (int q = gs; q < ge; ++q) esum += myE[q];
        int bin = -1;
        if (seag) bin = 0;
        else {
          const double Em = esum / (double)(ge - gs);
          if (Em < sp.EFmin) bin = 0;
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int c = 0; c < nc; ++c) {
            double v = 0.0;
            for (int q = gs; q < ge; ++q) v += myT[(size_t)q * nc + c];
            fx_add_double(sh + 2 * (bin * nc + c), v, sh + 2 * nh);
          }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (hist && shist) fx_flush(sh, nh, hist);
}

// ---------------------------------------------------------------------------------------
// Orbital moment, Morb_Hpm (formula/covariant.py:375-449): non-additive, so the trace over
// inn = [0, n), out = [n, nw) is needed at every group border n (calculators/static.py:109-117).
// The trace splits into pair functions of bands (m in inn, l in out / n' in inn):
//   T(n) = sum_{m<n} [ sum_{l>=n} F(m,l) + sum_{n'<n} G(m,n') + H(m) ]
//        = sum_{m<n} [ sum_{l>=n} (F - G)(m,l) + Gtot(m) + H(m) ]
// with (component g, (a,b) = ((1,2),(2,0),(0,1))[g], D_ml = -V_ml/(E_m - E_l)):
//   F = 2Re[-i D^a_ml E_l D^b_lm - D^a_ml B^b_lm + D^b_ml B^a_lm]                  (Morb_H)
//     + E_m 2Re[-i D^a_ml D^b_lm - D^a_ml A^b_lm + D^b_ml A^a_lm]                   (E_m Omega)
//   G = (E_n' + E_m) 2Re[-i A^a_mn' A^b_n'm],   H = Re C^g_mm + E_m Re O^g_mm.
// Lane m walks n downwards keeping the running suffix sum; one warp reduction per n gives T(n).
// Group values T(ge) - T(gs) are binned like the Omega kernel.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void berry_morb_kernel(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar,
                                  int iV, int iA, int iO, int iB, int iC, int nw, int nk, int L, int G, WbgScan sp,
                                  int internal_terms, int external_terms, wbg_u64* __restrict__ hist, int shist,
                                  BandSel bs) {
  typedef typename C2<T>::t V;
  extern __shared__ double smb[];
  const int nh = 3 * sp.nEF;  // histogram entries [nEF][3], fixed point (shared or global)
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);         // [G][nw]
  double* Tn = Es + G * nw;                              // [G][nw+1][3]
  int* start = reinterpret_cast<int*>(Tn + 3 * G * (nw + 1));  // [G][nw]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = Tn + 3 * grp * (nw + 1);
  int* myS = start + grp * nw;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
    for (int i = lane; i < nw; i += L) myE[i] = E[kk * nw + i];
    __syncwarp();
    for (int i = lane; i < nw; i += L) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    __syncwarp();
    int bandmax;
    if (bs.sel) {
      bandmax = sel_bandmax(bs.sel + kk * nw, nw, lane, L);
    } else {
      int below = 0, f0 = nw;
      for (int n = lane; n < nw; n += L) {
        below += myE[n] < sp.EFmin;
        if (myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) f0 = min(f0, n);
        }
      }
      below = group_sum_i(below, L);
      f0 = group_min_i(f0, L);
      bandmax = min(below, f0);
    }
    const V* Xk = Xbar + kk * nFbar * nw2;
    // per band: Gtot + H (constant part) and running suffix of F - G
    const int nb_lane = (nw + L - 1) / L;  // bands per lane (<= WBG_BAND_MAXPER)
    double cst[WBG_BAND_MAXPER][3], run[WBG_BAND_MAXPER][3];
    for (int q = 0; q < nb_lane; ++q) {
      const int m = lane + q * L;
      for (int g = 0; g < 3; ++g) { cst[q][g] = 0.0; run[q][g] = 0.0; }
      if (m >= nw || !external_terms) continue;
      const double Em = myE[m];
      for (int np = 0; np < nw; ++np) {
        const double w = myE[np] + Em;
#pragma unroll
        for (int g = 0; g < 3; ++g) {
          const int al = (g + 1) % 3, be = (g + 2) % 3;
          V acc = cmul(Xk[(iA + al) * nw2 + m * nw + np], Xk[(iA + be) * nw2 + np * nw + m]);
          cst[q][g] += w * 2.0 * (double)acc.y;  // 2 Re(-i acc) = 2 Im(acc)
        }
      }
#pragma unroll
      for (int g = 0; g < 3; ++g)
        cst[q][g] += (double)Xk[(iC + g) * nw2 + m * nw + m].x + Em * (double)Xk[(iO + g) * nw2 + m * nw + m].x;
    }
    for (int n = nw; n >= 1; --n) {
      double part[3] = {0.0, 0.0, 0.0};
      for (int q = 0; q < nb_lane; ++q) {
        const int m = lane + q * L;
        if (m >= n) continue;
        if (n < nw) {
          const int l = n;  // add (F - G)(m, l=n) to the running suffix sum
          const double Em = myE[m], El = myE[l];
          const double dE = Em - El;
          const T dinv = fabs(dE) < 1e-7 ? T(0) : recip_gap<T>(dE);
          V Dml[3], Dlm[3], Blm[3], Alm[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            Dml[a] = cscale(Xk[(iV + a) * nw2 + m * nw + l], -dinv);
            Dlm[a] = cscale(Xk[(iV + a) * nw2 + l * nw + m], dinv);
            Blm[a] = external_terms ? Xk[(iB + a) * nw2 + l * nw + m] : czero<V>();
            Alm[a] = external_terms ? Xk[(iA + a) * nw2 + l * nw + m] : czero<V>();
          }
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            double f = 0.0;
            if (internal_terms) {
              const V dd = cmul(Dml[al], Dlm[be]);  // 2Re(-i x) = 2 Im(x)
              f += 2.0 * (El + Em) * (double)dd.y;
            }
            if (external_terms) {
              V xb = csub(cmul(Dml[be], Blm[al]), cmul(Dml[al], Blm[be]));
              V xa = csub(cmul(Dml[be], Alm[al]), cmul(Dml[al], Alm[be]));
              f += 2.0 * ((double)xb.x + Em * (double)xa.x);
              const V aa = cmul(Xk[(iA + al) * nw2 + m * nw + l], Xk[(iA + be) * nw2 + l * nw + m]);
              f -= (El + Em) * 2.0 * (double)aa.y;  // minus G(m, l)
            }
            run[q][g] += f;
          }
        }
#pragma unroll
        for (int g = 0; g < 3; ++g) part[g] += run[q][g] + cst[q][g];
      }
      for (int g = 0; g < 3; ++g) {
        const double t = group_sum_d(part[g], L);
        if (lane == 0) myT[n * 3 + g] = t;
      }
    }
    if (lane == 0)
      for (int g = 0; g < 3; ++g) myT[g] = 0.0;  // T(0): empty inner set
    __syncwarp();
    if (valid && bs.P) {  // group values T(ge) - T(gs), per band (the sea on band 0)
      for (int n = lane; n < nw; n += L) {
        double v[3] = {0.0, 0.0, 0.0};
        if (n < bandmax) {
          if (n == 0)
            for (int g = 0; g < 3; ++g) v[g] = myT[bandmax * 3 + g] - myT[g];
        } else if (bs.sel[k * nw + n] == 1) {
          int gs = n, ge = n + 1;
          while (!myS[gs]) --gs;
          while (ge < nw && !myS[ge]) ++ge;
          for (int g = 0; g < 3; ++g) v[g] = (myT[ge * 3 + g] - myT[gs * 3 + g]) / (double)(ge - gs);
        }
        for (int g = 0; g < 3; ++g) bs.P[(k * nw + n) * 3 + g] = v[g];
      }
    } else if (valid) {
      for (int n = lane; n < nw; n += L) {
        int gs = -1, ge = -1;
        bool sea = false;
        if (n == 0 && bandmax > 0) { gs = 0; ge = bandmax; sea = true; }
        else if (n >= bandmax && myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { gs = n; ge = g1; }
        }
        if (gs < 0) continue;
        double esum = 0.0;
        for (int q = gs; q < ge; ++q) esum += myE[q];
        int bin = -1;
        if (sea) bin = 0;
        else {
          const double Em = esum / (double)(ge - gs);
          if (Em < sp.EFmin) bin = 0;
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int g = 0; g < 3; ++g) fx_add_double(sh + 2 * (bin * 3 + g), myT[ge * 3 + g] - myT[gs * 3 + g], sh + 2 * nh);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (hist && shist) fx_flush(sh, nh, hist);
}

// ---------------------------------------------------------------------------------------
// Berry-curvature dipole, DerOmega (formula/covariant.py:212-259), additive, 3x3 per group.
// For band m of group G (inn = G, out = the rest), with D_xy = -V_xy/(E_x - E_y):
//   dD_lm^{bd} = -[W^{bd}_lm + sum_{p notin G}(V^b_lp D^d_pm + V^d_lp D^b_pm)
//                            - sum_{q in G}(D^b_lq V^d_qm + D^d_lq V^b_qm)] / (E_l - E_m)
//   dD_ml^{ad} = -[W^{ad}_ml + sum_{p in G}(V^a_mp D^d_pl + V^d_mp D^a_pl)
//                            - sum_{q notin G}(D^a_mq V^d_ql + D^d_mq V^a_ql)] / (E_m - E_l)
//   dA_lm^{bd} = dAc^{bd}_lm - sum_{q in G} D^d_lq A^b_qm + sum_{p notin G} A^b_lp D^d_pm
//   dA_n'm^{bd} = dAc^{bd}_n'm - sum_{l notin G} D^d_n'l A^b_lm + sum_{l notin G} A^b_n'l D^d_lm
//   dO_mm^{cd} = dOc^{cd}_mm - sum_{l notin G} D^d_ml O^c_lm + sum_{l notin G} O^c_ml D^d_lm
// (elementary.py:55-70 DerDcov, formula.py:95-118 Matrix_GenDer_ln) and
//   S^{cd} = 1/2 dO^{cd}_mm + sum_{(s,a,b)} [ -i s sum_l D^a_ml dD^{bd}_lm
//            - s sum_l D^a_ml dA^{bd}_lm - s sum_l dD^{ad}_ml A^b_lm - i s sum_n' A^a_mn' dA^{bd}_n'm ]
// over (s,a,b) in {(+1, alpha_c, beta_c), (-1, beta_c, alpha_c)}; the group value is
// sum_{m in G} 2 Re S^{cd}.  hist is [nEF][3][3] (c, d) -- the calculator swaps c and d.
// ---------------------------------------------------------------------------------------
template <typename T, typename VS = typename C2<T>::t>
__global__ void berry_deromega_kernel(const double* __restrict__ E, const VS* __restrict__ Xbar,
                                      int nFbar, int iV, int iA, int iO, int iW, int idA, int idO, int nw, int nk,
                                      int L, int G, int table, WbgScan sp, int internal_terms, int external_terms,
                                      wbg_u64* __restrict__ hist, int shist, BandSel bs) {
  typedef typename C2<T>::t V;
  extern __shared__ double smb[];
  const int nh = 9 * sp.nEF;  // histogram entries [nEF][9], fixed point (shared or global)
  wbg_u64* sh = shist ? reinterpret_cast<wbg_u64*>(smb) : hist;
  double* Es = smb + (shist ? fx_words(nh) : 0);      // [G][nw]
  double* tv = Es + G * nw;                           // [G][nw][9]
  T* dinvS = reinterpret_cast<T*>(tv + 9 * G * nw);   // [G][nw][nw] when table != 0
  int* start = reinterpret_cast<int*>(dinvS + (table ? (size_t)G * nw * nw : 0));  // [G][nw]
  if (shist) fx_zero(sh, nh);
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = tv + 9 * grp * nw;
  T* myDinv = dinvS + (size_t)grp * nw * nw;
  int* myS = start + grp * nw;
  const long long nw2 = (long long)nw * nw;
  for (long long base = (long long)blockIdx.x * G; base < nk; base += (long long)gridDim.x * G) {
    const long long k = base + grp;
    const bool valid = k < nk;
    const long long kk = valid ? k : nk - 1;
    for (int i = lane; i < nw; i += L) myE[i] = E[kk * nw + i];
    __syncwarp();
    for (int i = lane; i < nw; i += L) myS[i] = (i == 0) || (myE[i] - myE[i - 1] > sp.degen_thresh);
    if (table)
      for (int idx = lane; idx < nw * nw; idx += L) {  // dinv(x, y) = 1/(E_x - E_y), 0 below 1e-7
        const int x = idx / nw, y = idx % nw;
        const double dE = myE[x] - myE[y];
        myDinv[idx] = fabs(dE) < 1e-7 ? Arith<T>::from(0.0) : recip_gap<T>(dE);
      }
    __syncwarp();
    int bandmax;
    if (bs.sel) {
      bandmax = sel_bandmax(bs.sel + kk * nw, nw, lane, L);
    } else {
      int below = 0, f0 = nw;
      for (int n = lane; n < nw; n += L) {
        below += myE[n] < sp.EFmin;
        if (myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) f0 = min(f0, n);
        }
      }
      below = group_sum_i(below, L);
      f0 = group_min_i(f0, L);
      bandmax = min(below, f0);
    }
    const VS* Xk = Xbar + kk * nFbar * nw2;
#define XV(a, x, y) ld_c<V>(Xk[(iV + (a)) * nw2 + (x) * nw + (y)])
#define XA(a, x, y) ld_c<V>(Xk[(iA + (a)) * nw2 + (x) * nw + (y)])
#define XO(a, x, y) ld_c<V>(Xk[(iO + (a)) * nw2 + (x) * nw + (y)])
#define XW(a, b, x, y) ld_c<V>(Xk[(iW + 3 * (a) + (b)) * nw2 + (x) * nw + (y)])
#define XdA(b, d, x, y) ld_c<V>(Xk[(idA + 3 * (b) + (d)) * nw2 + (x) * nw + (y)])
#define XdO(c, d, x, y) ld_c<V>(Xk[(idO + 3 * (c) + (d)) * nw2 + (x) * nw + (y)])
    // 1/(E_x - E_y) from the table, or recomputed when the table does not fit in shared memory
    auto dinv = [&](int x, int y) -> T {
      if (table) return myDinv[x * nw + y];
      const double dE = myE[x] - myE[y];
      return fabs(dE) < 1e-7 ? Arith<T>::from(0.0) : recip_gap<T>(dE);
    };
#define DV(a, x, y) cscale(XV(a, x, y), -dinv((x), (y)))
    for (int m = lane; m < nw; m += L) {
      int gs = m, ge = m + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      bool ingroup;
      if (m < bandmax) { gs = 0; ge = bandmax; ingroup = true; }
      else ingroup = bs.sel ? bs.sel[kk * nw + m] == 1 : (myE[ge - 1] >= sp.EFmin && myE[gs] <= sp.EFmax);
      double val[9];
      for (int i = 0; i < 9; ++i) val[i] = 0.0;
      if (ingroup) {
        for (int l = 0; l < nw; ++l) {
          if (l >= gs && l < ge) continue;
          const T dlm = dinv(l, m);  // 1/(E_l - E_m)
          V dDlm[9], dDml[9], dAlm[9];
          for (int i = 0; i < 9; ++i) { dDlm[i] = czero<V>(); dDml[i] = czero<V>(); dAlm[i] = czero<V>(); }
          for (int p = 0; p < nw; ++p) {
            const bool inG = (p >= gs && p < ge);
            V Vlp[3], Vpm[3], Vmp[3], Vpl[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) { Vlp[a] = XV(a, l, p); Vpm[a] = XV(a, p, m); Vmp[a] = XV(a, m, p); Vpl[a] = XV(a, p, l); }
            if (!inG) {
              // dD_lm: + V^b_lp D^d_pm ; dD_ml: - D^a_mp V^d_pl ; dA_lm: + A^b_lp D^d_pm
              const T dpm = dinv(p, m), dmp = dinv(m, p);
              V Dpm[3], Dmp[3], Alp[3];
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                Dpm[a] = cscale(Vpm[a], -dpm);
                Dmp[a] = cscale(Vmp[a], -dmp);
                Alp[a] = external_terms ? XA(a, l, p) : czero<V>();
              }
#pragma unroll
              for (int b = 0; b < 3; ++b)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  cmac(dDlm[3 * b + d], Vlp[b], Dpm[d]);
                  cmsub(dDml[3 * b + d], Dmp[b], Vpl[d]);
                  cmac(dAlm[3 * b + d], Alp[b], Dpm[d]);
                }
            } else {
              // dD_lm: - D^b_lp V^d_pm ; dD_ml: + V^a_mp D^d_pl ; dA_lm: - D^d_lp A^b_pm
              const T dlp = dinv(l, p), dpl = dinv(p, l);
              V Dlp[3], Dpl[3], Apm[3];
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                Dlp[a] = cscale(Vlp[a], -dlp);
                Dpl[a] = cscale(Vpl[a], -dpl);
                Apm[a] = external_terms ? XA(a, p, m) : czero<V>();
              }
#pragma unroll
              for (int b = 0; b < 3; ++b)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  cmsub(dDlm[3 * b + d], Dlp[b], Vpm[d]);
                  cmac(dDml[3 * b + d], Vmp[b], Dpl[d]);
                  cmsub(dAlm[3 * b + d], Dlp[d], Apm[b]);
                }
            }
          }
#pragma unroll
          for (int i = 0; i < 9; ++i) {
            dDlm[i] = cdone(dDlm[i]);
            dDml[i] = cdone(dDml[i]);
            dAlm[i] = cdone(dAlm[i]);
          }
          const T dml = dinv(m, l);  // 1/(E_m - E_l)
          // symmetrise in (b, d) (the bracket is symmetric, W = d_b d_d H too) and scale
#pragma unroll
          for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int d = b; d < 3; ++d) {
              const V t1 = cadd(cadd(dDlm[3 * b + d], dDlm[3 * d + b]), XW(b, d, l, m));
              const V t2 = cadd(cadd(dDml[3 * b + d], dDml[3 * d + b]), XW(b, d, m, l));
              dDlm[3 * b + d] = cscale(t1, -dlm);
              dDml[3 * b + d] = cscale(t2, -dml);
            }
#pragma unroll
          for (int b = 1; b < 3; ++b)
#pragma unroll
            for (int d = 0; d < b; ++d) { dDlm[3 * b + d] = dDlm[3 * d + b]; dDml[3 * b + d] = dDml[3 * d + b]; }
          if (external_terms) {
#pragma unroll
            for (int b = 0; b < 3; ++b)
#pragma unroll
              for (int d = 0; d < 3; ++d) dAlm[3 * b + d] = cadd(dAlm[3 * b + d], XdA(b, d, l, m));
          }
          V Dml[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) Dml[a] = DV(a, m, l);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const int al = (c + 1) % 3, be = (c + 2) % 3;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              double acc = 0.0;
              for (int t = 0; t < 2; ++t) {
                const double sg = t == 0 ? 1.0 : -1.0;
                const int a = t == 0 ? al : be, b = t == 0 ? be : al;
                if (internal_terms) acc += sg * to_dbl(cmul(Dml[a], dDlm[3 * b + d]).y);  // Re(-i s x) = s Im x
                if (external_terms) {
                  acc -= sg * to_dbl(cmul(Dml[a], dAlm[3 * b + d]).x);
                  acc -= sg * to_dbl(cmul(dDml[3 * a + d], XA(b, l, m)).x);
                }
              }
              if (external_terms) {  // 1/2 dO_mm: - D^d_ml O^c_lm + O^c_ml D^d_lm
                const V Dlm_d = DV(d, l, m);
                acc += 0.5 * (to_dbl(cmul(Dml[d], XO(c, l, m)).x) * -1.0 + to_dbl(cmul(XO(c, m, l), Dlm_d).x));
              }
              val[3 * c + d] += 2.0 * acc;
            }
          }
        }
        if (external_terms) {
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) val[3 * c + d] += to_dbl(XdO(c, d, m, m).x);  // 2 Re(1/2 dOc_mm)
          // -i s sum_{n' in G} A^a_mn' dA^{bd}_n'm
          for (int np = gs; np < ge; ++np) {
            V dAn[9];
#pragma unroll
            for (int b = 0; b < 3; ++b)
#pragma unroll
              for (int d = 0; d < 3; ++d) dAn[3 * b + d] = XdA(b, d, np, m);
            for (int l = 0; l < nw; ++l) {
              if (l >= gs && l < ge) continue;
              V Dnl[3], Dlm[3], Alm[3], Anl[3];
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                Dnl[a] = DV(a, np, l);
                Dlm[a] = DV(a, l, m);
                Alm[a] = XA(a, l, m);
                Anl[a] = XA(a, np, l);
              }
#pragma unroll
              for (int b = 0; b < 3; ++b)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  cmsub(dAn[3 * b + d], Dnl[d], Alm[b]);
                  cmac(dAn[3 * b + d], Anl[b], Dlm[d]);
                }
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) dAn[i] = cdone(dAn[i]);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const int al = (c + 1) % 3, be = (c + 2) % 3;
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                const double x1 = to_dbl(cmul(XA(al, m, np), dAn[3 * be + d]).y);
                const double x2 = to_dbl(cmul(XA(be, m, np), dAn[3 * al + d]).y);
                val[3 * c + d] += 2.0 * (x1 - x2);  // 2 Re(-i s A dA) = 2 s Im(A dA)
              }
            }
          }
        }
      }
      for (int i = 0; i < 9; ++i) myT[m * 9 + i] = val[i];
    }
#undef XV
#undef XA
#undef XO
#undef XW
#undef XdA
#undef XdO
#undef DV
    __syncwarp();
    if (valid && bs.P) {
      emit_band_values(bs.P, k, nw, 9, lane, L, bandmax, bs.sel + k * nw, myS, myT, 9);
    } else if (valid) {
      for (int n = lane; n < nw; n += L) {
        int gs = -1, ge = -1;
        bool sea = false;
        if (n == 0 && bandmax > 0) { gs = 0; ge = bandmax; sea = true; }
        else if (n >= bandmax && myS[n]) {
          int g1 = n + 1;
          while (g1 < nw && !myS[g1]) ++g1;
          if (myE[g1 - 1] >= sp.EFmin && myE[n] <= sp.EFmax) { gs = n; ge = g1; }
        }
        if (gs < 0) continue;
        double v[9], esum = 0.0;
        for (int i = 0; i < 9; ++i) v[i] = 0.0;
        for (int q = gs; q < ge; ++q) {
          for (int i = 0; i < 9; ++i) v[i] += myT[q * 9 + i];
          esum += myE[q];
        }
        int bin = -1;
        if (sea) bin = 0;
        else {
          const double Em = esum / (double)(ge - gs);
          if (Em < sp.EFmin) bin = 0;
          else if (Em <= sp.EFmax) bin = (int)ceil((Em - sp.EFmin) / sp.dEF);
        }
        if (bin >= 0 && bin < sp.nEF)
          for (int i = 0; i < 9; ++i) fx_add_double(sh + 2 * (bin * 9 + i), v[i], sh + 2 * nh);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  if (hist && shist) fx_flush(sh, nh, hist);
}

// cumulative sum over Fermi levels and normalisation: out[ie][c] = scale * sum_{j<=ie} hist[j][c],
// hist in the fixed-point layout of wbgpu_fixed.cuh; NaN throughout when a contribution was not finite
__global__ void scan_finalize_kernel(const wbg_u64* __restrict__ hist, int nEF, int ncomp, double scale,
                                     double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncomp) return;
  const bool bad = hist[2 * (size_t)nEF * ncomp] != 0ull;
  double s = 0.0;
  for (int ie = 0; ie < nEF; ++ie) {
    const size_t e = (size_t)ie * ncomp + c;
    s += fx_value(hist[2 * e], hist[2 * e + 1]);
    out[e] = bad ? nan("") : s * scale;
  }
}

// Shared memory of a formula kernel with an nh-entry histogram and `rest` bytes of other
// per-block data: the fixed-point histogram sits in shared memory when both fit in one block
// (shist = 1), else the kernel adds into the global histogram directly (shist = 0).
size_t hist_smem(int nh, size_t rest, int& shist) {
  const size_t h = fx_words((size_t)nh) * 8;
  shist = h + rest <= 220 * 1024 ? 1 : 0;
  return (shist ? h : 0) + rest;
}

int lanes_for(int n) {
  int L = 1;
  while (L < n && L < 32) L <<= 1;
  return L < 4 ? 4 : L;
}

// k-points per block of rotate_tiled that fit: a power of two, at most 256 threads and 200 KB of
// shared memory per block
bool tiled_kpoints_fit(int kb, int tpk, size_t per_k) {
  return kb >= 1 && !(kb & (kb - 1)) && kb * tpk <= 256 && (size_t)kb * per_k <= 200 * 1024;
}

template <typename T, typename VO = typename C2<T>::t>
int launch_rotate(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                  int nFrot, void* Xbar, int nw, int nk, cudaStream_t stream) {
  typedef typename C2<T>::t V;
  if (nw > 64) {  // row panels: the per-k matrices no longer fit in shared memory together
    if (nw > 4 * 256 / (PANEL_RP / 4)) return WBG_ERR_SIZE;  // threads = (RP/4) * ceil(nw/4) <= 256
    const int np = (nw + PANEL_RP - 1) / PANEL_RP;
    const int threads = (PANEL_RP / 4) * ((nw + 3) / 4);
    const size_t sm = ((size_t)PANEL_RP * (nw + 1) + (size_t)PANEL_KC * nw + PANEL_KC * PANEL_RP) * sizeof(V);
    const long long blocks = (long long)np * nFrot * nk;
    if (sm > 220 * 1024 || blocks > 0x7fffffffll) return WBG_ERR_SIZE;
    cudaFuncSetAttribute(rotate_panel<T, VO>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    rotate_panel<T, VO><<<(unsigned)blocks, threads, sm, stream>>>((const V*)U, strideU, (const V*)X, nFin, fsel,
                                                                   herm, nFrot, (VO*)Xbar, nw, nk);
    return wbg_cuda_status(cudaGetLastError());
  }
  if (nw % 4 == 0 && nw >= 8) {
    const int tpk = (nw / 4) * (nw / 4);
    const size_t per_k = ((size_t)nw * nw * 2 + (size_t)nw * (nw + 1)) * sizeof(V);
    int KB = 1;
    while (KB * 2 * tpk <= 256 && (KB * 2) * per_k <= 64 * 1024) KB *= 2;
    if (KB * per_k <= 200 * 1024) {
      const int t = wbg_tuned(WBG_TUNE_ROTATE_KPOINTS, sizeof(T) == 8 ? 1 : 0, nw);
      if (t > 0 && tiled_kpoints_fit(t, tpk, per_k)) KB = t;
      cudaFuncSetAttribute(rotate_tiled<T, VO>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      rotate_tiled<T, VO><<<(nk + KB - 1) / KB, KB * tpk, KB * per_k, stream>>>(
          (const V*)U, strideU, (const V*)X, nFin, fsel, herm, nFrot, (VO*)Xbar, nw, nk, KB);
      return wbg_cuda_status(cudaGetLastError());
    }
  }
  const size_t sm = 3 * (size_t)nw * nw * sizeof(V);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  // rotate_kernel writes every element (treats herm == 2 like 1): the full Hermitian part is a
  // valid superset of the diagonal-only request
  cudaFuncSetAttribute(rotate_kernel<T, VO>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  rotate_kernel<T, VO><<<nk, 256, sm, stream>>>((const V*)U, strideU, (const V*)X, nFin, fsel, herm, nFrot, (VO*)Xbar,
                                                nw);
  return wbg_cuda_status(cudaGetLastError());
}

}  // namespace

int wbg_rotate_run(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                   int nFrot, void* Xbar, int nw, int nk, int fp64, cudaStream_t stream) {
  if (nw < 1 || nk < 1 || nFrot < 1 || !U || !X || !Xbar || !fsel || !herm) return WBG_ERR_ARG;
  // tensor cores (3xTF32) for the FP32 path at nw = 32 (unless the tuner chose the CUDA cores);
  // the kernel reads X in 16-byte pieces
  const int engine = wbg_tuned(WBG_TUNE_ROTATE_ENGINE, fp64 ? 1 : 0, nw);
  if (wbg_rotate_tc_supported(nw, fp64, nFrot) && (reinterpret_cast<uintptr_t>(X) & 15) == 0 && engine != 2)
    return wbg_rotate_tc_run(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream, engine != 1);
  if (fp64 < 0 || fp64 > 2) return WBG_ERR_ARG;
  if (fp64 == 2)  // double-float U and X, products in double-float, Xbar rounded to complex64
    return launch_rotate<df64, float2>(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream);
  if (fp64) return launch_rotate<double>(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream);
  return launch_rotate<float>(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream);
}

int wbg_rotate_tune_candidates(int param, int nw, int variant, int* values, int capacity) {
  int count = 0;
  if (param == WBG_TUNE_ROTATE_ENGINE) {
    if (wbg_rotate_tc_supported(nw, variant, 1))
      for (int v = 1; v <= 3 && count < capacity; ++v) values[count++] = v;
    return count;
  }
  if (param != WBG_TUNE_ROTATE_KPOINTS || nw % 4 != 0 || nw < 8 || nw > 64) return 0;
  // the tiled kernel serves this (nw, precision) when its built-in block fits (launch_rotate)
  const int tpk = (nw / 4) * (nw / 4);
  const size_t per_k = ((size_t)nw * nw * 2 + (size_t)nw * (nw + 1)) * (variant ? 16 : 8);
  int KB = 1;
  while (KB * 2 * tpk <= 256 && (KB * 2) * per_k <= 64 * 1024) KB *= 2;
  if (KB * per_k > 200 * 1024) return 0;
  for (int v = 1; v <= 256; v *= 2)
    if (tiled_kpoints_fit(v, tpk, per_k) && count < capacity) values[count++] = v;
  return count;
}

int wbg_berry_omega_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                        const WbgScan* sp_in, int internal_terms, int external_terms, void* hist, int fp64,
                        cudaStream_t stream, double* tab, const signed char* sel, double* P) {
  const BandSel bs{sel, P};
  if (nw < 1 || nk < 1 || !sp_in || !E || !Xbar || (!sel) != (!P)) return WBG_ERR_ARG;
  if (!sel && (sp_in->nEF < 1 || (!hist && !tab) || !(sp_in->dEF > 0.0))) return WBG_ERR_ARG;
  if (iV < 0 || iV + 3 > nFbar) return WBG_ERR_ARG;
  if (external_terms && (iA < 0 || iA + 3 > nFbar || iO < 0 || iO + 3 > nFbar)) return WBG_ERR_ARG;
  if (fp64 < 0 || fp64 > 2) return WBG_ERR_ARG;
  WbgScan spv = *sp_in;
  if (sel) { spv.nEF = 0; hist = nullptr; tab = nullptr; }  // per-band values: no histogram
  const WbgScan* sp = &spv;
  if (fp64 == 2 && nw <= 128 && !tab && !sel) {  // FP32, exactly Hermitian V and A: column-per-lane kernel
    const int C = (nw + 31) / 32;
    const int G = 4;  // k-points (warps) per block
    int shist = 0;
    const size_t sm = hist_smem(3 * sp->nEF, (size_t)G * 32 * C * (8 + 24 + 8 + 4), shist);
    if (sm > 220 * 1024) return WBG_ERR_SIZE;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    long long nblk = (nk + G - 1) / G;
    const long long cap = (long long)sms * 16;
    if (nblk > cap) nblk = cap;
    void (*kern)(const double*, const float2*, int, int, int, int, int, int, int, WbgScan, int, int, wbg_u64*, int) =
        C == 1 ? berry_omega_cols<1> : C == 2 ? berry_omega_cols<2> : C == 3 ? berry_omega_cols<3> : berry_omega_cols<4>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    kern<<<(int)nblk, 32 * G, sm, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, iO, nw, nk, G, *sp, internal_terms,
                                           external_terms, (wbg_u64*)hist, shist);
    return wbg_cuda_status(cudaGetLastError());
  }
  if (fp64 == 2) fp64 = 0;  // the general FP32 kernel does not need the symmetry
  const int L = lanes_for(nw);
  const int G = 128 / L;
  int shist = 0;
  const size_t sm = hist_smem(3 * sp->nEF, (size_t)G * nw * (8 + 24 + 8 + 4), shist);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  const long long cap = (long long)sms * 8;
  if (nblk > cap) nblk = cap;
  if (fp64) {
    cudaFuncSetAttribute(berry_omega_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_omega_kernel<double><<<(int)nblk, G * L, sm, stream>>>(E, (const double2*)Xbar, nFbar, iV, iA, iO, nw, nk, L,
                                                                 G, *sp, internal_terms, external_terms, (wbg_u64*)hist, shist, tab,
                                                                 bs);
  } else {
    cudaFuncSetAttribute(berry_omega_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_omega_kernel<float><<<(int)nblk, G * L, sm, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, iO, nw, nk, L,
                                                                G, *sp, internal_terms, external_terms, (wbg_u64*)hist, shist, tab,
                                                                 bs);
  }
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_berry_scan_run(const double* E, const void* Xbar, int nFbar, int iV, int iW, int nw, int nk,
                       const WbgScan* sp_in, int formula, int sea, void* hist, int fp64, cudaStream_t stream,
                       const signed char* sel, double* P, const wbg_dynamic_spec* spin) {
  const BandSel bs{sel, P};
  if (nw < 1 || nk < 1 || !sp_in || !E || (!sel) != (!P)) return WBG_ERR_ARG;
  if (!sel && (sp_in->nEF < 1 || !hist || !(sp_in->dEF > 0.0))) return WBG_ERR_ARG;
  WbgScan spv = *sp_in;
  if (sel) { spv.nEF = 0; hist = nullptr; }
  const WbgScan* sp = &spv;
  const bool plain = formula >= WBG_FORMULA_IDENTITY && formula <= WBG_FORMULA_VELVEL;
  if (!plain && formula != WBG_FORMULA_DIAG && formula != WBG_FORMULA_VELVELVEL && formula != WBG_FORMULA_SPIN_OMEGA)
    return WBG_ERR_ARG;
  if (formula != WBG_FORMULA_IDENTITY && (!Xbar || iV < 0 || iV + 3 > nFbar)) return WBG_ERR_ARG;
  if (formula == WBG_FORMULA_INVMASS && (iW < 0 || iW + 9 > nFbar)) return WBG_ERR_ARG;
  wbg_dynamic_spec fs = {};
  if (formula == WBG_FORMULA_SPIN_OMEGA) {  // the spin current's fields (as wbg_dynamic's SHC)
    if (!spin) return WBG_ERR_ARG;
    fs = *spin;
    auto ok = [&](int first, int n) { return first >= 0 && first + n <= nFbar; };
    const int K = fs.formula;
    if (K < WBG_DYN_SHC_SIMPLE || K > WBG_DYN_SHC_RYOO || (fs.external_terms != 0 && fs.external_terms != 1))
      return WBG_ERR_ARG;
    if (!ok(fs.V, 3) || !ok(fs.S, 3) || (fs.external_terms && !ok(fs.A, 3))) return WBG_ERR_ARG;
    if (K != WBG_DYN_SHC_SIMPLE && !fs.external_terms) return WBG_ERR_ARG;
    if (K == WBG_DYN_SHC_QIAO && !(ok(fs.SH, 3) && ok(fs.SR, 9) && ok(fs.SHR, 9))) return WBG_ERR_ARG;
    if (K == WBG_DYN_SHC_RYOO && !(ok(fs.SA, 9) && ok(fs.SHA, 9))) return WBG_ERR_ARG;
  }
  const int nc = scan_ncomp(formula);
  const int L = lanes_for(nw);
  const int G = 128 / L;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  if (nblk > (long long)sms * 8) nblk = (long long)sms * 8;
#define WBG_SCAN(TT, NCM)                                                                                          \
  do {                                                                                                             \
    int shist = 0;                                                                                                 \
    const size_t sm = hist_smem(nc * sp->nEF, (size_t)G * nw * (8 + 8 * NCM + 4), shist);                         \
    if (sm > 220 * 1024) return WBG_ERR_SIZE;                                                                      \
    cudaFuncSetAttribute(berry_scan_kernel<TT, NCM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);     \
    berry_scan_kernel<TT, NCM><<<(int)nblk, G * L, sm, stream>>>(E, (const typename C2<TT>::t*)Xbar, nFbar, iV, iW, \
                                                                 nw, nk, L, G, *sp, formula, sea, (wbg_u64*)hist,  \
                                                                 shist, bs, fs);                                   \
  } while (0)
  if (nc == 27) {
    if (fp64) WBG_SCAN(double, 27);
    else WBG_SCAN(float, 27);
  } else {
    if (fp64) WBG_SCAN(double, 9);
    else WBG_SCAN(float, 9);
  }
#undef WBG_SCAN
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_berry_product_run(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                          const WbgScan* sp_in, int sea, void* hist, int fp64, cudaStream_t stream,
                          const signed char* sel, double* P) {
  const BandSel bs{sel, P};
  if (nw < 1 || nk < 1 || !sp_in || !E || !Xbar || !spec || (!sel) != (!P) || (fp64 != 0 && fp64 != 1))
    return WBG_ERR_ARG;
  if (!sel && (sp_in->nEF < 1 || !hist || !(sp_in->dEF > 0.0))) return WBG_ERR_ARG;
  const wbg_product_spec ps = *spec;
  if (ps.nfactors < 1 || ps.nfactors > 3) return WBG_ERR_ARG;
  auto ok = [&](int first, int n) { return first >= 0 && first + n <= nFbar; };
  int nc = 1;
  for (int i = 0; i < ps.nfactors; ++i) {
    const int f = ps.factor[i];
    if (f == WBG_FACTOR_VEL) {
      if (!ok(ps.V, 3)) return WBG_ERR_ARG;
    } else if (f == WBG_FACTOR_SPIN) {
      if (!ok(ps.S, 3)) return WBG_ERR_ARG;
    } else if (f == WBG_FACTOR_OMEGA) {
      if (!ok(ps.V, 3) || (ps.external_terms && !(ok(ps.A, 3) && ok(ps.O, 3)))) return WBG_ERR_ARG;
    } else if (f == WBG_FACTOR_MASS) {
      if (!ok(ps.V, 3) || !ok(ps.W, 9)) return WBG_ERR_ARG;
    } else if (f == WBG_FACTOR_DERSPIN) {
      if (!ok(ps.V, 3) || !ok(ps.S, 3) || !ok(ps.dS, 9)) return WBG_ERR_ARG;
    } else if (f == WBG_FACTOR_HPLUS) {
      if (!ok(ps.V, 3) || (ps.external_terms && !(ok(ps.A, 3) && ok(ps.O, 3) && ok(ps.B, 3) && ok(ps.C, 3))))
        return WBG_ERR_ARG;
    } else {
      return WBG_ERR_ARG;
    }
    if ((f == WBG_FACTOR_OMEGA || f == WBG_FACTOR_HPLUS) &&
        ((ps.internal_terms != 0 && ps.internal_terms != 1) || (ps.external_terms != 0 && ps.external_terms != 1)))
      return WBG_ERR_ARG;
    nc *= (f == WBG_FACTOR_MASS || f == WBG_FACTOR_DERSPIN) ? 9 : 3;
  }
  WbgScan spv = *sp_in;
  if (sel) { spv.nEF = 0; hist = nullptr; }
  const int L = lanes_for(nw);
  const size_t per_group = (size_t)nw * (8 + 8 * (size_t)nc + 8 + 4);
  int G = 128 / L;
  while (G > 1 && (size_t)G * per_group > 96 * 1024) G /= 2;
  int shist = 0;
  const size_t sm = hist_smem(nc * spv.nEF, (size_t)G * per_group, shist);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  if (nblk > (long long)sms * 8) nblk = (long long)sms * 8;
  if (fp64) {
    auto kern = berry_product_kernel<double, double2>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    kern<<<(int)nblk, G * L, sm, stream>>>(E, (const double2*)Xbar, nFbar, ps, nc, nw, nk, L, G, spv, sea,
                                           (wbg_u64*)hist, shist, bs);
  } else {
    auto kern = berry_product_kernel<double, float2>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    kern<<<(int)nblk, G * L, sm, stream>>>(E, (const float2*)Xbar, nFbar, ps, nc, nw, nk, L, G, spv, sea,
                                           (wbg_u64*)hist, shist, bs);
  }
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_berry_morb_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iB, int iC, int nw,
                       int nk, const WbgScan* sp_in, int internal_terms, int external_terms, void* hist, int fp64,
                       cudaStream_t stream, const signed char* sel, double* P) {
  const BandSel bs{sel, P};
  if (nw < 1 || nk < 1 || !sp_in || !E || !Xbar || (!sel) != (!P)) return WBG_ERR_ARG;
  if (!sel && (sp_in->nEF < 1 || !hist || !(sp_in->dEF > 0.0))) return WBG_ERR_ARG;
  WbgScan spv = *sp_in;
  if (sel) { spv.nEF = 0; hist = nullptr; }
  const WbgScan* sp = &spv;
  if (iV < 0 || iV + 3 > nFbar) return WBG_ERR_ARG;
  if (external_terms && (iA < 0 || iA + 3 > nFbar || iO < 0 || iO + 3 > nFbar || iB < 0 || iB + 3 > nFbar ||
                         iC < 0 || iC + 3 > nFbar))
    return WBG_ERR_ARG;
  const int L = lanes_for(nw);
  if ((nw + L - 1) / L > WBG_BAND_MAXPER) return WBG_ERR_SIZE;
  const int G = 128 / L;
  int shist = 0;
  const size_t sm =
      hist_smem(3 * sp->nEF, (size_t)G * nw * 8 + (size_t)G * (nw + 1) * 24 + (size_t)G * nw * 4, shist);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  const long long cap = (long long)sms * 8;
  if (nblk > cap) nblk = cap;
  if (fp64) {
    cudaFuncSetAttribute(berry_morb_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_morb_kernel<double><<<(int)nblk, G * L, sm, stream>>>(E, (const double2*)Xbar, nFbar, iV, iA, iO, iB, iC,
                                                                nw, nk, L, G, *sp, internal_terms, external_terms,
                                                                (wbg_u64*)hist, shist, bs);
  } else {
    cudaFuncSetAttribute(berry_morb_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_morb_kernel<float><<<(int)nblk, G * L, sm, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, iO, iB, iC, nw,
                                                               nk, L, G, *sp, internal_terms, external_terms,
                                                               (wbg_u64*)hist, shist, bs);
  }
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_berry_deromega_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iW, int idA,
                           int idO, int nw, int nk, const WbgScan* sp_in, int internal_terms, int external_terms,
                           void* hist, int fp64, cudaStream_t stream, const signed char* sel, double* P) {
  const BandSel bs{sel, P};
  if (nw < 1 || nk < 1 || !sp_in || !E || !Xbar || (!sel) != (!P) || fp64 < 0 || fp64 > 2) return WBG_ERR_ARG;
  if (!sel && (sp_in->nEF < 1 || !hist || !(sp_in->dEF > 0.0))) return WBG_ERR_ARG;
  WbgScan spv = *sp_in;
  if (sel) { spv.nEF = 0; hist = nullptr; }
  const WbgScan* sp = &spv;
  if (iV < 0 || iV + 3 > nFbar || iW < 0 || iW + 9 > nFbar) return WBG_ERR_ARG;
  if (external_terms && (iA < 0 || iA + 3 > nFbar || iO < 0 || iO + 3 > nFbar || idA < 0 || idA + 9 > nFbar ||
                         idO < 0 || idO + 9 > nFbar))
    return WBG_ERR_ARG;
  const int L = lanes_for(nw);
  int G = 64 / L > 0 ? 64 / L : 1;
  const size_t tsz = fp64 ? 8 : 4;
  // per-block data besides the histogram: energies, traces, group starts and the 1/dE table
  auto rest = [&](int g, int table) {
    return (size_t)g * nw * (8 + 72 + 4) + (table ? (size_t)g * nw * nw * tsz : 0);
  };
  const size_t hbytes = fx_words((size_t)9 * sp->nEF) * 8;
  auto smem = [&](int g, int table) { return hbytes + rest(g, table); };
  int table = 1;  // k-point groups per block shrink before the 1/dE table is dropped
  while (G > 1 && smem(G, 1) > 220 * 1024) G /= 2;
  if (smem(G, 1) > 220 * 1024) table = 0;
  int shist = 0;
  if (smem(G, table) > 220 * 1024) {  // the histogram goes global before anything else gives way
    G = 64 / L > 0 ? 64 / L : 1;
    table = 1;
    while (G > 1 && rest(G, 1) > 220 * 1024) G /= 2;
    if (rest(G, 1) > 220 * 1024) table = 0;
  }
  const size_t sm = hist_smem(9 * sp->nEF, rest(G, table), shist);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  const long long cap = (long long)sms * 8;
  if (nblk > cap) nblk = cap;
  if (fp64 == 1) {
    cudaFuncSetAttribute(berry_deromega_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_deromega_kernel<double><<<(int)nblk, G * L, sm, stream>>>(E, (const double2*)Xbar, nFbar, iV, iA, iO, iW,
                                                                    idA, idO, nw, nk, L, G, table, *sp, internal_terms,
                                                                    external_terms, (wbg_u64*)hist, shist, bs);
  } else if (fp64 == 2) {  // complex64 Xbar, double-float arithmetic
    cudaFuncSetAttribute(berry_deromega_kernel<df64, float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         220 * 1024);
    berry_deromega_kernel<df64, float2><<<(int)nblk, G * L, sm, stream>>>(
        E, (const float2*)Xbar, nFbar, iV, iA, iO, iW, idA, idO, nw, nk, L, G, table, *sp, internal_terms,
        external_terms, (wbg_u64*)hist, shist, bs);
  } else {
    cudaFuncSetAttribute(berry_deromega_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_deromega_kernel<float><<<(int)nblk, G * L, sm, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, iO, iW, idA,
                                                                   idO, nw, nk, L, G, table, *sp, internal_terms,
                                                                   external_terms, (wbg_u64*)hist, shist, bs);
  }
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_scan_finalize_run(const void* hist, int nEF, int ncomp, double scale, double* out, cudaStream_t stream) {
  if (nEF < 1 || ncomp < 1 || !hist || !out) return WBG_ERR_ARG;
  scan_finalize_kernel<<<(ncomp + 31) / 32, 32, 0, stream>>>((const wbg_u64*)hist, nEF, ncomp, scale, out);
  return wbg_cuda_status(cudaGetLastError());
}
