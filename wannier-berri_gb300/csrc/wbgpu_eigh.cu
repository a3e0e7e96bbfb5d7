// Batched Hermitian eigensolver (stage 2 of the path): H(k) -> E_K (ascending), UU_K.
//
// Replaces np.linalg.eigh in data_K/data_K.py:211-218 (E_K, UU_K) applied to
// HH_K = 1/2 (H + H^dagger) (fourier/fft.py:183-186, data_K/data_K_R.py:24-26).
//
// GB300 runs FP64 at ~1.9 DFMA/clk/SM and a warp instruction costs the same whether
// one lane or 32 lanes are active, so each phase is mapped so that every lane does
// useful work:
//   1. eigh_tridiag : Householder reduction to real tridiagonal T = Q^dagger H Q,
//                     lower triangle only, mirrored row pairs per lane (shared memory).
//   2. eigh_ql      : implicit QL (Wilkinson shift) eigenvalues of T, one thread per matrix.
//   3. eigh_vectors : inverse iteration on T (partial-pivot LU), one lane per eigenvector,
//                     modified Gram-Schmidt inside clusters, back-transform by the
//                     Householder reflectors (U = Q Z).
// The three kernels are templates over the real type R of the solve: native double, or
// df64 (double-float on the FP32 pipe, 48-bit significand) for the mixed-precision path.
// The back-transform runs in precision TU (double or float).
#include <float.h>
#include "wbgpu_common.cuh"
#include "wbgpu_df64.cuh"
#include "wbgpu_eigh.cuh"
#include "wbgpu_tune.cuh"

namespace {

template <typename R>
WBG_D R group_sum(R v, int L) {
  for (int off = L / 2; off > 0; off >>= 1) v = v + shfl_xor(v, off);
  return v;
}

template <typename R>
WBG_D typename C2<R>::t from_c64(double2 a) {
  typename C2<R>::t r;
  r.x = Arith<R>::from(a.x);
  r.y = Arith<R>::from(a.y);
  return r;
}
// 1/2 (a + conj(b)) of two input elements, input either complex128 or double-float complex
template <typename R>
WBG_D typename C2<R>::t herm_avg(double2 a, double2 b) {
  return from_c64<R>(make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y)));
}
template <typename R>
WBG_D typename C2<R>::t herm_avg(cdf a, cdf b) {
  typename C2<R>::t r;
  const df64 half = df_from_f(0.5f);
  r.x = (a.x + b.x) * half;
  r.y = (a.y - b.y) * half;
  return r;
}
template <>
WBG_D float2 herm_avg<float>(cdf a, cdf b) {  // the FP32 solve of the refined mode
  const df64 half = df_from_f(0.5f);
  const df64 x = (a.x + b.x) * half, y = (a.y - b.y) * half;
  return make_float2(x.hi + x.lo, y.hi + y.lo);
}

// Element (i, j <= i) of a matrix given by its lower triangle; the diagonal is taken real.
template <typename R>
WBG_D typename C2<R>::t lower_elem(double2 a, bool diag) {
  return from_c64<R>(make_double2(a.x, diag ? 0.0 : a.y));
}
template <typename R>
WBG_D typename C2<R>::t lower_elem(cdf a, bool diag) {
  if (diag) a.y = Arith<R>::from(0.0);
  return a;
}
template <>
WBG_D float2 lower_elem<float>(cdf a, bool diag) {
  return make_float2(a.x.hi + a.x.lo, diag ? 0.0f : a.y.hi + a.y.lo);
}

// Rounding of a solver real into the back-transform precision.  df64 -> float adds the two
// halves on the FP32 pipe (|lo| <= ulp(hi)/2, so hi + lo is the correctly rounded float up
// to a tie); no value passes through the FP64 pipe.
template <typename TU> WBG_D TU to_tu(double x);
template <> WBG_D double to_tu<double>(double x) { return x; }
template <> WBG_D float to_tu<float>(double x) { return (float)x; }
template <typename TU> WBG_D TU to_tu(df64 x);
template <> WBG_D float to_tu<float>(df64 x) { return x.hi + x.lo; }
template <> WBG_D df64 to_tu<df64>(df64 x) { return x; }
template <typename TU, typename CR> WBG_D typename C2<TU>::t to_tu_c(CR a) {
  typename C2<TU>::t r;
  r.x = to_tu<TU>(a.x);
  r.y = to_tu<TU>(a.y);
  return r;
}
// the stored eigenvectors: the back-transform type, or FP32 rounded from a more precise one
template <typename VO, typename VU> WBG_D VO store_u(VU a) { return a; }
template <> WBG_D float2 store_u<float2, double2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
template <> WBG_D float2 store_u<float2, cdf>(cdf a) { return make_float2(a.x.hi + a.x.lo, a.y.hi + a.y.lo); }
template <typename V> WBG_D bool cnonzero(V a) { return a.x != 0 || a.y != 0; }
template <> WBG_D bool cnonzero<cdf>(cdf a) { return a.x.hi != 0.0f || a.y.hi != 0.0f; }

// ---------------------------------------------------------------------------------------
// 1. Householder tridiagonalisation.  grid: ceil(nk/G) blocks of G*L threads.
// Only the lower triangle of the Hermitian matrix is kept, packed row by row
// (element (i, j <= i) at i(i+1)/2 + j): half the shared memory of a full matrix, so twice
// the matrices per SM.  Lane l of a group owns the mirrored row pairs
// (2Lt + l, 2Lt + 2L-1-l), so the triangular rank-2 update is balanced across lanes;
// L = max(4, pow2ceil(n)/2), i.e. two matrices share a warp for 16 < n <= 32.
// Outputs: d[k][i], e[k][i] (e[n-1] = 0) in the solver type R; Vh[k][c][i] (v of reflector
// c, v_{c+1}=1, zeros for i<=c) and tau[k][c] rounded to the back-transform type TV.
// ---------------------------------------------------------------------------------------
// Lazy multiply-add chains (df_lazy_fma of wbgpu_df64.cuh for double-float; an ordinary fma
// for double), renormalised once at the end of the chain by lz_done.
WBG_D void lz_fma(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
WBG_D float lz_done(float acc) { return acc; }
WBG_D void lz_fma(double& acc, double a, double b) { acc = fma(a, b, acc); }
WBG_D double lz_done(double acc) { return acc; }
WBG_D void lz_fma(df64& acc, df64 a, df64 b) { df_lazy_fma(acc, a, b); }
WBG_D df64 lz_done(df64 acc) { return df_lazy_done(acc); }
template <typename CR> WBG_D void lz_cfma(CR& acc, const CR& a, const CR& b) {  // acc += a b
  lz_fma(acc.x, a.x, b.x);
  lz_fma(acc.x, -a.y, b.y);
  lz_fma(acc.y, a.x, b.y);
  lz_fma(acc.y, a.y, b.x);
}
template <typename CR> WBG_D void lz_cfmac(CR& acc, const CR& a, const CR& b) {  // acc += conj(a) b
  lz_fma(acc.x, a.x, b.x);
  lz_fma(acc.x, a.y, b.y);
  lz_fma(acc.y, a.x, b.y);
  lz_fma(acc.y, -a.y, b.x);
}
template <typename CR> WBG_D CR lz_cdone(CR a) {
  a.x = lz_done(a.x);
  a.y = lz_done(a.y);
  return a;
}

WBG_D int owned_row(int t, int half, int l, int L) {  // half 0: 2Lt + l, half 1: 2Lt + 2L-1-l
  return 2 * L * t + (half ? 2 * L - 1 - l : l);
}
WBG_D int tri(int i) { return (i * (i + 1)) >> 1; }  // start of packed row i

template <typename R, typename HIn, typename TV>
__global__ void eigh_tridiag(const HIn* __restrict__ H, long long strideK, int n, int nk, int L, int G, int lowerIn,
                             typename C2<TV>::t* __restrict__ Vh, typename C2<TV>::t* __restrict__ tauOut,
                             R* __restrict__ dOut, R* __restrict__ eOut) {
  typedef typename C2<R>::t CR;
  typedef typename C2<TV>::t CV;
  typedef Arith<R> A;
  extern __shared__ unsigned char smt[];
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  long long k = (long long)blockIdx.x * G + grp;
  const bool valid = k < nk;
  if (!valid) k = nk - 1;  // redundant work keeps every lane of the warp in the same control flow
  const int ntri = tri(n);
  CR* Am = reinterpret_cast<CR*>(smt) + (size_t)grp * (ntri + 2 * n);
  CR* vs = Am + ntri;
  CR* ws = vs + n;
  const HIn* Hk = H + k * strideK;
  for (int idx = lane; idx < n * n; idx += L) {
    const int i = idx / n, j = idx % n;
    if (j <= i)
      Am[tri(i) + j] = lowerIn ? lower_elem<R>(Hk[i * n + j], i == j) : herm_avg<R>(Hk[i * n + j], Hk[j * n + i]);
  }
  __syncwarp();
  const R zero = A::from(0.0), one = A::from(1.0), mhalf = A::from(-0.5);
  const int T = (n + 2 * L - 1) / (2 * L);
  for (int c = 0; c < n - 1; ++c) {
    R xn = zero;
    for (int t = 0; t < T; ++t)
      for (int h = 0; h < 2; ++h) {
        const int i = owned_row(t, h, lane, L);
        if (i < n && i >= c + 2) { const CR x = Am[tri(i) + c]; xn = fma(x.x, x.x, fma(x.y, x.y, xn)); }
      }
    xn = group_sum(xn, L);
    const CR alpha = Am[tri(c + 1) + c];
    R beta, tr = zero, ti = zero;
    CR scale = czero<CR>();
    if (xn == zero && alpha.y == zero) {
      beta = alpha.x;  // H = I
    } else {
      const R nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn);
      beta = alpha.x >= zero ? -nrm : nrm;
      const R rb = one / beta;
      tr = (beta - alpha.x) * rb;
      ti = -alpha.y * rb;
      // scale = 1 / (alpha - beta)
      const R ar = alpha.x - beta, ai = alpha.y;
      const R rden = one / (ar * ar + ai * ai);
      scale.x = ar * rden;
      scale.y = -ai * rden;
    }
    CR tau;
    tau.x = tr;
    tau.y = ti;
    // executed unconditionally (tau = 0 makes it a no-op) so that every lane of the warp
    // reaches the same __syncwarp / shuffle calls when several matrices share a warp
    for (int t = 0; t < T; ++t)
      for (int h = 0; h < 2; ++h) {
        const int i = owned_row(t, h, lane, L);
        if (i < n) {
          if (i == c + 1) { CR v1; v1.x = one; v1.y = zero; vs[i] = v1; Am[tri(i) + c] = v1; }
          else if (i >= c + 2) { const CR v = cmul(Am[tri(i) + c], scale); vs[i] = v; Am[tri(i) + c] = v; }
        }
      }
    __syncwarp();
    // p = tau * A v over the full Hermitian row: lower part A[i][j], upper part conj(A[j][i])
    R dr = zero, di = zero;
    for (int t = 0; t < T; ++t)
      for (int h = 0; h < 2; ++h) {
        const int i = owned_row(t, h, lane, L);
        if (i < n && i >= c + 1) {
          // four independent accumulators (two per part of the row): the double-float
          // multiply-adds are long dependent chains, so the lane needs several in flight
          CR acc = czero<CR>(), acc1 = czero<CR>(), acc2 = czero<CR>(), acc3 = czero<CR>();
          const CR* Ai = Am + tri(i);
          int j = c + 1;
          for (; j < i; j += 2) {
            lz_cfma(acc, Ai[j], vs[j]);
            lz_cfma(acc1, Ai[j + 1], vs[j + 1]);
          }
          if (j == i) lz_cfma(acc, Ai[j], vs[j]);
          j = i + 1;
          int idx = tri(i + 1) + i;
          for (; j + 1 < n; j += 2) {
            lz_cfmac(acc2, Am[idx], vs[j]);
            lz_cfmac(acc3, Am[idx + j + 1], vs[j + 1]);
            idx += 2 * j + 3;
          }
          if (j < n) lz_cfmac(acc2, Am[idx], vs[j]);
          acc = lz_cdone(acc);
          acc1 = lz_cdone(acc1);
          acc2 = lz_cdone(acc2);
          acc3 = lz_cdone(acc3);
          acc.x = (acc.x + acc1.x) + (acc2.x + acc3.x);
          acc.y = (acc.y + acc1.y) + (acc2.y + acc3.y);
          const CR p = cmul(tau, acc);
          ws[i] = p;
          const CR v = vs[i];
          dr = fma(p.x, v.x, fma(p.y, v.y, dr));  // conj(p) v
          di = fma(p.x, v.y, fma(-p.y, v.x, di));
        }
      }
    dr = group_sum(dr, L);
    di = group_sum(di, L);
    // alpha2 = -1/2 tau (w^dagger v)
    CR dd;
    dd.x = dr;
    dd.y = di;
    const CR a2 = cscale(cmul(tau, dd), mhalf);
    for (int t = 0; t < T; ++t)
      for (int h = 0; h < 2; ++h) {
        const int i = owned_row(t, h, lane, L);
        if (i < n && i >= c + 1) cfma(ws[i], a2, vs[i]);
      }
    __syncwarp();
    // lower-triangle rank-2 update: A[i][j] -= v_i conj(w_j) + w_i conj(v_j), c+1 <= j <= i
    for (int t = 0; t < T; ++t)
      for (int h = 0; h < 2; ++h) {
        const int i = owned_row(t, h, lane, L);
        if (i < n && i >= c + 1) {
          const CR vi = vs[i], wi = ws[i];
          CR* Ai = Am + tri(i);
#pragma unroll 2
          for (int j = c + 1; j <= i; ++j) {
            CR a = Ai[j];
            const CR vj = vs[j], wj = ws[j];
            lz_fma(a.x, -vi.x, wj.x);
            lz_fma(a.x, -vi.y, wj.y);
            lz_fma(a.x, -wi.x, vj.x);
            lz_fma(a.x, -wi.y, vj.y);
            lz_fma(a.y, -vi.y, wj.x);
            lz_fma(a.y, vi.x, wj.y);
            lz_fma(a.y, -wi.y, vj.x);
            lz_fma(a.y, wi.x, vj.y);
            Ai[j] = lz_cdone(a);
          }
        }
      }
    __syncwarp();
    if (valid) {
      const bool refl = (tr != zero || ti != zero);
      for (int i = lane; i < n; i += L)
        Vh[(k * n + c) * n + i] = (refl && i >= c + 1) ? to_tu_c<TV>(Am[tri(i) + c]) : czero<CV>();
      if (lane == 0) {
        tauOut[k * n + c] = to_tu_c<TV>(tau);
        eOut[k * n + c] = beta;
        dOut[k * n + c] = Am[tri(c) + c].x;
      }
    }
    __syncwarp();
  }
  if (valid && lane == 0) {
    dOut[k * n + n - 1] = Am[tri(n - 1) + n - 1].x;
    eOut[k * n + n - 1] = zero;
    tauOut[k * n + n - 1] = czero<CV>();
  }
  if (valid)
    for (int i = lane; i < n; i += L) Vh[(k * n + n - 1) * n + i] = czero<CV>();
}

// ---------------------------------------------------------------------------------------
// 2. Implicit QL eigenvalues of the real symmetric tridiagonal (d, e), thread per matrix.
// d and e of thread t live in shared memory at [i * blockDim + t] (conflict-free, no
// local-memory traffic).
// ---------------------------------------------------------------------------------------
template <typename R>
__global__ void eigh_ql(const R* __restrict__ dIn, const R* __restrict__ eIn, int n, int nk, double* __restrict__ Eout,
                        int* __restrict__ errflag) {
  typedef Arith<R> A;
  extern __shared__ unsigned char smq[];
  const int B = blockDim.x;
  const long long k = (long long)blockIdx.x * B + threadIdx.x;
  if (k >= nk) return;
  R* ds = reinterpret_cast<R*>(smq) + threadIdx.x;
  R* es = ds + (size_t)n * B;
  auto d = [&](int i) -> R& { return ds[i * B]; };
  auto e = [&](int i) -> R& { return es[i * B]; };
  const R zero = A::from(0.0), one = A::from(1.0), two = A::from(2.0), eps = A::eps();
  for (int i = 0; i < n; ++i) { d(i) = dIn[k * n + i]; e(i) = eIn[k * n + i]; }
  e(n - 1) = zero;
  bool ok = true;
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        const R dd = fabs(d(m)) + fabs(d(m + 1));
        if (fabs(e(m)) <= eps * dd) break;
      }
      if (m != l) {
        if (iter++ >= 60) { ok = false; break; }
        R g = (d(l + 1) - d(l)) / (two * e(l));
        R r = sqrt(fma(g, g, one));
        g = d(m) - d(l) + e(l) / (g + copysign(r, g));
        R s = one, c = one, p = zero;
        bool underflow = false;
        for (int i = m - 1; i >= l; --i) {
          const R f = s * e(i);
          const R b = c * e(i);
          // Givens rotation: one sqrt and one reciprocal (f, g are O(|T|): no overflow concern)
          r = sqrt(fma(f, f, g * g));
          e(i + 1) = r;
          if (r == zero) { d(i + 1) = d(i + 1) - p; e(m) = zero; underflow = true; break; }
          const R rinv = one / r;
          s = f * rinv;
          c = g * rinv;
          g = d(i + 1) - p;
          r = (d(i) - g) * s + two * c * b;
          p = s * r;
          d(i + 1) = g + p;
          g = c * r - b;
        }
        if (underflow) continue;
        d(l) = d(l) - p;
        e(l) = g;
        e(m) = zero;
      }
    } while (m != l);
    if (!ok) break;
  }
  if (!ok) atomicOr(errflag, WBG_FLAG_QL_NOCONV);
  // ascending insertion sort
  for (int i = 1; i < n; ++i) {
    const R x = d(i);
    int j = i - 1;
    while (j >= 0 && d(j) > x) { d(j + 1) = d(j); --j; }
    d(j + 1) = x;
  }
  for (int i = 0; i < n; ++i) Eout[k * n + i] = A::to(d(i));
}

WBG_D double hash_uniform(unsigned int a, unsigned int b) {
  unsigned int h = a * 2654435761u ^ (b + 0x9e3779b9u + (a << 6) + (a >> 2));
  h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
  return (double)(h & 0xffffff) / (double)0x800000 - 1.0;  // [-1, 1)
}

// ---------------------------------------------------------------------------------------
// 3. Eigenvectors: inverse iteration on T (real type R, two solves from a pseudo-random
//    start), clusters re-orthogonalised, U = Q Z.
// grid: ceil(nk/G) blocks of G*L threads; lane j computes eigenvectors j, j+L, ...
// The back-transform by the Householder reflectors runs in precision TU, one reflector at a
// time staged in shared memory for all lanes.  Shared memory per group: Z [n][n], d, e,
// lam [n] (type R), then U[n][n] and the staged reflector [n], complex(TU).  The iterate of
// lane j lives in column j of Z.  When complex(TU) and R have the same size (df64 solve,
// float vectors) U overlays Z: element (i, j) is converted in place by the lane that owns
// column j, so the group needs half the shared memory.  When complex(TU) is twice R (vectors
// in the precision of the solve) U starts where Z starts and the conversion runs row by row.
// ---------------------------------------------------------------------------------------
template <typename R, typename TU>
constexpr bool kUOverlaysZ = sizeof(typename C2<TU>::t) == sizeof(R);
// complex(TU) twice the size of R (double-float or FP64 vectors from a solve of the same type): U
// holds Z in the first half of its region, converted row by row from the last (row i of U covers
// rows 2i and 2i+1 of Z, which are read by then), so the group needs U's region only
template <typename R, typename TU>
constexpr bool kUWideOverlay = sizeof(typename C2<TU>::t) == 2 * sizeof(R);

template <typename R, typename TU, typename VO>
__global__ void eigh_vectors(const typename C2<TU>::t* __restrict__ Vh, const typename C2<TU>::t* __restrict__ tauIn,
                             const R* __restrict__ dIn, const R* __restrict__ eIn, const double* __restrict__ E, int n,
                             int nk, int L, int G, int CW, VO* __restrict__ Uout, long long strideU) {
  typedef typename C2<TU>::t VU;
  typedef Arith<R> A;
  extern __shared__ unsigned char smv[];
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  long long k = (long long)blockIdx.x * G + grp;
  const bool valid = k < nk;
  if (!valid) k = nk - 1;
  const size_t zbytes = (((size_t)n * n + 3 * n) * sizeof(R) + 15) / 16 * 16;
  const size_t ubytes = kUOverlaysZ<R, TU> ? 0 : ((size_t)n * CW * sizeof(VU) + 15) / 16 * 16;
  const size_t vbytes = ((size_t)n * sizeof(VU) + 15) / 16 * 16;
  const bool wide = kUWideOverlay<R, TU> && CW == n;
  const size_t regbytes = wide ? (zbytes > ubytes ? zbytes : ubytes) : zbytes + ubytes;
  unsigned char* gbase = smv + (size_t)grp * (regbytes + vbytes);
  R* Zs = reinterpret_cast<R*>(gbase);  // Z(i,j) = Zs[i*n + j]
  R* ds = Zs + n * n;
  R* es = ds + n;
  R* lam = es + n;
  VU* Us = (kUOverlaysZ<R, TU> || wide) ? reinterpret_cast<VU*>(gbase)
                                         : reinterpret_cast<VU*>(gbase + zbytes);  // [i][j-c0]
  VU* vsh = reinterpret_cast<VU*>(gbase + regbytes);
  for (int i = lane; i < n; i += L) { ds[i] = dIn[k * n + i]; es[i] = eIn[k * n + i]; lam[i] = A::from(E[k * n + i]); }
  __syncwarp();
  const R zero = A::from(0.0), one = A::from(1.0);
  R tnorm = zero;
  for (int i = 0; i < n; ++i) tnorm = fmax(tnorm, fabs(ds[i]) + fabs(es[i]) + (i > 0 ? fabs(es[i - 1]) : zero));
  tnorm = fmax(tnorm, A::tiny_norm());
  const R tiny = A::pivot_floor() * tnorm;
  const R ortol = A::from(1e-5) * tnorm;
  const R pertol = A::from(10.0) * A::eps() * tnorm;
  // Per lane: reciprocal pivots and first super-diagonal of U (the only factors that cannot
  // be rebuilt), a row-swap bitmask; the iterate lives in column j of Z.
  R u0i[WBG_EIGH_NMAX], u1[WBG_EIGH_NMAX];
  for (int j = lane; j < n; j += L) {
    R shift = lam[j];
    for (int jj = j - 1; jj >= 0 && shift - lam[jj] < pertol; --jj) shift = lam[jj] + pertol * A::from((double)(j - jj));
    R* x = Zs + j;  // x[i * n]: column j of Z
    for (int i = 0; i < n; ++i) x[i * n] = A::from(hash_uniform((unsigned)j + 1u, (unsigned)i + 7u));
    for (int it = 0; it < 2; ++it) {  // the second solve squares the contamination left by the first
      // LU with partial pivoting of T - shift I, fused with x := L^{-1} P x.  Row i of U is
      // (1/u0i[i], u1[i], u2[i]); u2[i] = e[i+1] after a row swap at step i, else 0.
      unsigned int swp[(WBG_EIGH_NMAX + 31) / 32];
      for (int w = 0; w < (n + 31) / 32; ++w) swp[w] = 0u;
      R ca = ds[0] - shift, cb = n > 1 ? es[0] : zero, xc = x[0];
      for (int i = 0; i < n - 1; ++i) {
        const R ci = es[i], ai1 = ds[i + 1] - shift, bi1 = (i + 1 < n - 1) ? es[i + 1] : zero;
        const R xn = x[(i + 1) * n];
        if (fabs(ca) >= fabs(ci)) {
          if (fabs(ca) < tiny) ca = ca >= zero ? tiny : -tiny;
          const R rc = one / ca;
          const R mlt = ci * rc;
          u0i[i] = rc; u1[i] = cb;
          x[i * n] = xc;
          xc = xn - mlt * xc;
          ca = ai1 - mlt * cb;
          cb = bi1;
        } else {
          const R rc = one / ci;
          const R mlt = ca * rc;
          u0i[i] = rc; u1[i] = ai1;
          swp[i >> 5] |= 1u << (i & 31);
          x[i * n] = xn;
          xc = xc - mlt * xn;
          ca = cb - mlt * ai1;
          cb = -mlt * bi1;
        }
      }
      if (fabs(ca) < tiny) ca = ca >= zero ? tiny : -tiny;
      R xi1 = xc / ca, xi2 = zero;  // x[i+1], x[i+2] of the back substitution
      x[(n - 1) * n] = xi1;
      R amax = fabs(xi1);
      for (int i = n - 2; i >= 0; --i) {
        const R u2 = ((swp[i >> 5] >> (i & 31)) & 1u) && (i + 1 < n - 1) ? es[i + 1] : zero;
        const R xi = (x[i * n] - u1[i] * xi1 - u2 * xi2) * u0i[i];
        x[i * n] = xi;
        amax = fmax(amax, fabs(xi));
        xi2 = xi1;
        xi1 = xi;
      }
      // scale by the largest component before the 2-norm so squares cannot overflow
      const R ra = one / amax;
      R nrm = zero;
      for (int i = 0; i < n; ++i) { const R xs = x[i * n] * ra; x[i * n] = xs; nrm = fma(xs, xs, nrm); }
      nrm = rsqrt(nrm);
      for (int i = 0; i < n; ++i) x[i * n] = x[i * n] * nrm;
    }
  }
  __syncwarp();
  // modified Gram-Schmidt inside clusters (eigenvalues closer than ortol), in eigenvalue order
  bool anyc = false;
  for (int j = 1; j < n; ++j) anyc |= (lam[j] - lam[j - 1] < ortol);
  anyc = __any_sync(0xffffffffu, anyc);  // warp-uniform: groups sharing a warp run the same loop
  if (anyc) {
    for (int jp = 0; jp < n - 1; ++jp) {
      for (int j = lane; j < n; j += L) {
        if (j > jp) {
          bool same = true;
          for (int q = jp + 1; q <= j; ++q) same &= (lam[q] - lam[q - 1] < ortol);
          if (same) {
            R dot = zero;
            for (int i = 0; i < n; ++i) dot = fma(Zs[i * n + jp], Zs[i * n + j], dot);
            for (int i = 0; i < n; ++i) Zs[i * n + j] = Zs[i * n + j] - dot * Zs[i * n + jp];
            if (j == jp + 1) {
              R nrm = zero;
              for (int i = 0; i < n; ++i) nrm = fma(Zs[i * n + j], Zs[i * n + j], nrm);
              nrm = rsqrt(nrm);
              for (int i = 0; i < n; ++i) Zs[i * n + j] = Zs[i * n + j] * nrm;
            }
          }
        }
      }
      __syncwarp();
    }
  }
  // back-transform: u = H_0 H_1 ... H_{n-2} z  (precision TU), in chunks of CW columns (every
  // column is independent; CW < n only when a full U does not fit in shared memory)
  for (int c0 = 0; c0 < n; c0 += CW) {
    const int cw = min(CW, n - c0);
    if (wide) {  // U over Z: rows from the last, every lane's reads of a row before its writes
      for (int i = n - 1; i >= 0; --i) {
        constexpr int kQ = (WBG_EIGH_NMAX + 31) / 32;  // columns per lane (L >= min(n, 32))
        R zr[kQ];
#pragma unroll
        for (int q = 0; q < kQ; ++q)
          if (lane + q * L < n) zr[q] = Zs[i * n + lane + q * L];
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kQ; ++q)
          if (lane + q * L < n) {
            VU z = czero<VU>();
            z.x = to_tu<TU>(zr[q]);
            Us[i * n + lane + q * L] = z;
          }
        __syncwarp();
      }
    } else {
      for (int jj = lane; jj < cw; jj += L)
        for (int i = 0; i < n; ++i) {
          VU z = czero<VU>();
          z.x = to_tu<TU>(Zs[i * n + c0 + jj]);
          Us[i * CW + jj] = z;
        }
    }
    for (int c = n - 2; c >= 0; --c) {
      // every lane passes the same __syncwarp calls: groups sharing a warp have different tau
      const VU tau = tauIn[k * n + c];
      const bool act = cnonzero(tau);
      for (int i = c + 1 + lane; i < n; i += L) vsh[i] = Vh[(k * n + c) * n + i];
      __syncwarp();
      if (act)
        for (int jj = lane; jj < cw; jj += L) {
          // v^H u as two lazy chains (even and odd rows): in double-float a chain step costs one
          // FP32 add on its critical path, the error terms are summed once at the end
          VU sacc = czero<VU>(), sacc1 = czero<VU>();
          int i = c + 1;
          for (; i + 1 < n; i += 2) {
            lz_cfmac(sacc, vsh[i], Us[i * CW + jj]);
            lz_cfmac(sacc1, vsh[i + 1], Us[(i + 1) * CW + jj]);
          }
          if (i < n) lz_cfmac(sacc, vsh[i], Us[i * CW + jj]);
          sacc = lz_cdone(sacc);
          sacc1 = lz_cdone(sacc1);
          sacc.x = sacc.x + sacc1.x;
          sacc.y = sacc.y + sacc1.y;
          const VU ts = cmul(tau, sacc);
          for (int i = c + 1; i < n; ++i) {
            VU u = Us[i * CW + jj];
            const VU vv = vsh[i];
            u.x = u.x - (vv.x * ts.x - vv.y * ts.y);
            u.y = u.y - (vv.x * ts.y + vv.y * ts.x);
            Us[i * CW + jj] = u;
          }
        }
      __syncwarp();
    }
    if (valid)
      for (int idx = lane; idx < n * cw; idx += L) {
        const int i = idx / cw, jj = idx % cw;
        Uout[k * strideU + i * n + c0 + jj] = store_u<VO, VU>(Us[i * CW + jj]);
      }
    __syncwarp();
  }
}

int lanes_for(int n) {
  int L = 1;
  while (L < n && L < 32) L <<= 1;
  return L < 4 ? 4 : L;
}

// ---------------------------------------------------------------------------------------
// 4. Refinement of an FP32 eigendecomposition against the double-float H (WBG_EIGH_REFINE):
//    one step of the Ogita-Aishima iteration (T. Ogita, K. Aishima, "Iterative refinement for
//    symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35, 2018), with a
//    Rayleigh-Ritz step inside clusters of close eigenvalues.
// One warp per matrix, n <= 32; lane j owns eigenvector x_j of the FP32 solve (U, E):
//   r_j = H x_j - lambda_j x_j           H x_j in double-float, r rounded to FP32
//   C_ij = x_i^H r_j                      FP32 (|r| ~ 1e-6 |H|: the sum's rounding is far below
//                                         what the step needs)
//   lambda'_j = lambda_j + C_jj / |x_j|^2 + sum_{i unclustered} |C_ij|^2 / (lambda_j - lambda_i)
//          (the Rayleigh quotient of x_j and its second-order error, which the step removes
//          from the vector: ~ (u |H|)^2 / gap otherwise)
//   x'_j = x_j + sum_i x_i E_ij,  E_ij = C_ij / (lambda_j - lambda_i) when the two are more than
//          delta apart, -x_i^H x_j / 2 inside a cluster, E_jj = (1 - |x_j|^2) / 2
// (C_ij = x_i^H H x_j - lambda_j x_i^H x_j holds both the paper's S_ij and lambda_j R_ij.)
// A cluster is a run of eigenvalues whose consecutive gaps are at most delta (2^-8 of the
// largest |lambda|): its refined columns X_c are re-diagonalised by Rayleigh-Ritz,
// P = X_c^H H X_c (H X_c in double-float, the sums in FP64), X_c orthonormalised by
// Gc = X_c^H X_c = L L^H (Cholesky in FP64 from the FP32 columns), L^-1 P L^-H = V diag(mu) V^H
// by cyclic Jacobi in FP64, X_c <- X_c L^-H V, lambda_c <- mu.  A cluster of more than RF_MAXC is
// re-diagonalised in consecutive runs of RF_MAXC (exact where its eigenvalues are exactly
// degenerate) and flagged (WBG_FLAG_REFINE_WIDE).  From an FP32 solve the step gives eigenvalues
// to ~1e-13 |H| and eigenvectors to the complex64 rounding.
// ---------------------------------------------------------------------------------------
constexpr int RF_MAXC = 8;  // largest cluster re-diagonalised by Rayleigh-Ritz

WBG_D void lz_fma_mixed(df64& acc, df64 a, float b) {  // acc += a b (a double-float, b FP32), lazily
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  const float s = acc.hi + p;
  const float v = s - acc.hi;
  const float t = (acc.hi - (s - v)) + (p - v);
  acc.hi = s;
  acc.lo = acc.lo + (t + e);
}

// H(k) into shared memory as the packed lower triangle (row i from i (i + 1) / 2) of double-float
// complex: from the lower triangle of the input, or 1/2 (H + H^dagger) of the full matrix; the
// diagonal real.  One warp, n <= 32.
WBG_D cdf to_cdf(cdf a) { return a; }
WBG_D cdf to_cdf(double2 a) {
  cdf r;
  r.x = df_from(a.x);
  r.y = df_from(a.y);
  return r;
}
template <typename HIn>
WBG_D void stage_h(const HIn* Hk, int n, int lowerIn, cdf* Hs, int lane) {
  const df64 half = df_from_f(0.5f);
  for (int i = 0; i < n; ++i)
    if (lane <= i) {
      cdf a = to_cdf(Hk[i * n + lane]);
      if (!lowerIn) {
        const cdf b = to_cdf(Hk[lane * n + i]);
        a.x = (a.x + b.x) * half;
        a.y = (a.y - b.y) * half;
      }
      if (lane == i) a.y = df_from_f(0.0f);
      Hs[tri(i) + lane] = a;
    }
}
WBG_D cdf hs_elem(const cdf* Hs, int i, int m) {  // element (i, m) of the staged H
  if (m <= i) return Hs[tri(i) + m];
  cdf a = Hs[tri(m) + i];
  a.y = -a.y;
  return a;
}

// acc += h v (complex, h double-float, v FP32)
WBG_D void lz_cfma_mixed(df64& ar, df64& ai, const cdf& h, float2 v) {
  lz_fma_mixed(ar, h.x, v.x);
  lz_fma_mixed(ar, -h.y, v.y);
  lz_fma_mixed(ai, h.x, v.y);
  lz_fma_mixed(ai, h.y, v.x);
}
// acc += conj(h) v
WBG_D void lz_cfmac_mixed(df64& ar, df64& ai, const cdf& h, float2 v) {
  lz_fma_mixed(ar, h.x, v.x);
  lz_fma_mixed(ar, h.y, v.y);
  lz_fma_mixed(ai, h.x, v.y);
  lz_fma_mixed(ai, -h.y, v.x);
}

// m x m Hermitian A (row-major, FP64) -> diagonal (ascending), V <- its eigenvectors
// (columns): cyclic Jacobi, each rotation W = diag(1, e^{-i phi}) J on the pair (p, q) with
// a_pq = r e^{i phi} and J the real rotation that zeroes r (tangent t = sgn(th) /
// (|th| + sqrt(th^2 + 1)), th = (a_qq - a_pp) / 2r)
WBG_D void jacobi_herm(double2* A, double2* V, int m) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) V[i * m + j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, nrm = 0.0;
    for (int p = 0; p < m; ++p) {
      nrm += A[p * m + p].x * A[p * m + p].x;
      for (int q = p + 1; q < m; ++q) off += A[p * m + q].x * A[p * m + q].x + A[p * m + q].y * A[p * m + q].y;
    }
    if (off <= 1e-32 * nrm || off == 0.0) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double2 b = A[p * m + q];
        const double r = sqrt(b.x * b.x + b.y * b.y);
        if (r == 0.0) continue;
        const double2 ph = make_double2(b.x / r, -b.y / r);  // e^{-i phi}
        const double th = (A[q * m + q].x - A[p * m + p].x) / (2.0 * r);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        const double2 w00 = make_double2(c, 0.0), w01 = make_double2(s, 0.0);
        const double2 w10 = make_double2(-s * ph.x, -s * ph.y), w11 = make_double2(c * ph.x, c * ph.y);
        for (int u = 0; u < m; ++u) {  // A <- A W, V <- V W
          const double2 ap = A[u * m + p], aq = A[u * m + q];
          A[u * m + p] = cadd(cmul(ap, w00), cmul(aq, w10));
          A[u * m + q] = cadd(cmul(ap, w01), cmul(aq, w11));
          const double2 vp = V[u * m + p], vq = V[u * m + q];
          V[u * m + p] = cadd(cmul(vp, w00), cmul(vq, w10));
          V[u * m + q] = cadd(cmul(vp, w01), cmul(vq, w11));
        }
        for (int u = 0; u < m; ++u) {  // A <- W^H A
          const double2 ap = A[p * m + u], aq = A[q * m + u];
          A[p * m + u] = cadd(cmulc(w00, ap), cmulc(w10, aq));
          A[q * m + u] = cadd(cmulc(w01, ap), cmulc(w11, aq));
        }
        A[p * m + q] = make_double2(0.0, 0.0);
        A[q * m + p] = make_double2(0.0, 0.0);
        A[p * m + p].y = 0.0;
        A[q * m + q].y = 0.0;
      }
  }
  for (int i = 0; i < m; ++i) {  // ascending
    int b = i;
    for (int j = i + 1; j < m; ++j)
      if (A[j * m + j].x < A[b * m + b].x) b = j;
    if (b != i) {
      const double2 t = A[i * m + i];
      A[i * m + i] = A[b * m + b];
      A[b * m + b] = t;
      for (int r = 0; r < m; ++r) {
        const double2 v = V[r * m + i];
        V[r * m + i] = V[r * m + b];
        V[r * m + b] = v;
      }
    }
  }
}

WBG_D double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// shared memory of one matrix: X [32][32] complex64 (column j at stride 32: the FP32 solve,
// then the refined columns), H (packed lower triangle, double-float complex), lamd [32], the
// cluster's P (then W), Gc (then S), A and V [RF_MAXC^2] complex128, lamf [32], cluster starts [32]
constexpr size_t RF_X_BYTES = 32 * 32 * 8, RF_H_BYTES = 32 * 33 / 2 * 16, RF_PC_BYTES = RF_MAXC * RF_MAXC * 16;
constexpr size_t RF_GROUP_BYTES = RF_X_BYTES + RF_H_BYTES + 32 * 8 + 4 * RF_PC_BYTES + 32 * 4 + 32 * 4;

template <typename HIn>
__global__ void __launch_bounds__(64, 1) eigh_refine(const HIn* __restrict__ H, long long strideH, int n, int nk,
                                                  int lowerIn, float2* __restrict__ U, long long strideU,
                                                  double* __restrict__ E, int G, int* __restrict__ errflag,
                                                  const int* __restrict__ list, int* __restrict__ relist) {
  extern __shared__ __align__(16) unsigned char smr[];
  const int grp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // first step: matrix blockIdx.x G + grp; second step (list): the listed matrices
  long long k = (long long)blockIdx.x * G + grp;
  const long long cnt = list ? list[0] : nk;
  const bool valid = k < cnt;
  if (list && !valid) return;  // past the listed matrices: the warp leaves (no block-wide barrier here)
  if (!valid) k = nk - 1;       // a tail warp repeats the last matrix and writes nothing
  if (list) k = list[1 + k];
  unsigned char* base = smr + (size_t)grp * RF_GROUP_BYTES;
  float2* X = reinterpret_cast<float2*>(base);
  cdf* Hs = reinterpret_cast<cdf*>(base + RF_X_BYTES);
  double* lamd = reinterpret_cast<double*>(base + RF_X_BYTES + RF_H_BYTES);
  double2* Pc = reinterpret_cast<double2*>(lamd + 32);
  double2* Gc = Pc + RF_MAXC * RF_MAXC;
  double2* Ab = Gc + RF_MAXC * RF_MAXC;
  double2* Vb = Ab + RF_MAXC * RF_MAXC;
  float* lamf = reinterpret_cast<float*>(Vb + RF_MAXC * RF_MAXC);
  int* cstart = reinterpret_cast<int*>(lamf + 32);
  stage_h<HIn>(H + k * strideH, n, lowerIn, Hs, lane);
  for (int idx = lane; idx < n * n; idx += 32) X[(idx / n) * 32 + idx % n] = U[k * strideU + idx];
  for (int i = lane; i < n; i += 32) lamf[i] = (float)E[k * n + i];  // FP32 eigenvalues, exact
  __syncwarp();
  const int j = lane < n ? lane : n - 1;  // lanes past n repeat the last column (nothing written)
  float amax = 0.0f;
  for (int i = 0; i < n; ++i) amax = fmaxf(amax, fabsf(lamf[i]));
  const float delta = amax * 0x1p-8f;
  const float lj = lamf[j];
  const df64 mlj = df_from_f(-lj);
  float2 r[32];  // residual of column j
#pragma unroll
  for (int i0 = 0; i0 < 32; i0 += 4) {
    if (i0 < n) {
      df64 ar[4], ai[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) ar[t] = ai[t] = df_from_f(0.0f);
      // rows i0 .. i0 + 3 (past n: row n - 1, discarded): columns m <= i0 from the rows of the
      // triangle, m > i0 + 3 from its columns (conjugated), the three between element by element
      for (int m = 0; m <= i0; ++m) {
        const float2 v = X[m * 32 + j];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int i = i0 + t < n ? i0 + t : n - 1;
          lz_cfma_mixed(ar[t], ai[t], Hs[tri(i) + m], v);
        }
      }
      for (int m = i0 + 1; m < n && m <= i0 + 3; ++m) {
        const float2 v = X[m * 32 + j];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int i = i0 + t < n ? i0 + t : n - 1;
          lz_cfma_mixed(ar[t], ai[t], hs_elem(Hs, i, m), v);
        }
      }
      for (int m = i0 + 4; m < n; ++m) {
        const float2 v = X[m * 32 + j];
        const cdf* hm = Hs + tri(m) + i0;
#pragma unroll
        for (int t = 0; t < 4; ++t) lz_cfmac_mixed(ar[t], ai[t], hm[t], v);
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = i0 + t < n ? i0 + t : n - 1;
        const float2 xi = X[i * 32 + j];
        lz_fma_mixed(ar[t], mlj, xi.x);
        lz_fma_mixed(ai[t], mlj, xi.y);
        const df64 a = df_lazy_done(ar[t]), b = df_lazy_done(ai[t]);
        r[i0 + t] = i0 + t < n ? make_float2(a.hi + a.lo, b.hi + b.lo) : make_float2(0.0f, 0.0f);
      }
    } else {
#pragma unroll
      for (int t = 0; t < 4; ++t) r[i0 + t] = make_float2(0.0f, 0.0f);
    }
  }
  // cluster starts by the FP32 eigenvalues; lane j's column is in a cluster (of two or more)
  if (lane < n) cstart[lane] = lane == 0 || lamf[lane] - lamf[lane - 1] > delta;
  __syncwarp();
  const bool inc = lane < n && (!cstart[lane] || (lane + 1 < n && !cstart[lane + 1]));
  float2 xp[32];  // the correction x'_j - x_j (kept apart from x_j: one rounding at the end)
  float gj = 0.0f;  // |x_j|^2 (FP32: enters lambda' through C_jj / gj, C_jj ~ 1e-6 |H|)
#pragma unroll
  for (int m = 0; m < 32; ++m) {
    xp[m] = make_float2(0.0f, 0.0f);
    const float2 v = m < n ? X[m * 32 + j] : make_float2(0.0f, 0.0f);
    gj = fmaf(v.x, v.x, fmaf(v.y, v.y, gj));
  }
  double lnew = lj;
  float l2 = 0.0f;  // second-order part: the Rayleigh quotient of x_j errs by sum_i |C_ij|^2 / (lambda_i - lambda_j)
  float emax = 0.0f;  // largest correction of the column
  for (int i = 0; i < n; ++i) {
    float2 c0 = make_float2(0.0f, 0.0f), c1 = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int m = 0; m < 32; m += 2) {
      if (m < n) cfmac(c0, X[m * 32 + i], r[m]);
      if (m + 1 < n) cfmac(c1, X[(m + 1) * 32 + i], r[m + 1]);
    }
    const float2 c = make_float2(c0.x + c1.x, c0.y + c1.y);
    const float d = lj - lamf[i];
    const bool near = i != j && fabsf(d) <= delta;
    float2 g = make_float2(0.0f, 0.0f);
    if (__any_sync(0xffffffffu, near))  // same cluster: first-order orthogonalisation, E_ij = -G_ij / 2
      for (int m = 0; m < n; ++m) cfmac(g, X[m * 32 + i], X[m * 32 + j]);
    float2 e;
    if (i == j) {
      lnew = (double)lj + (double)(c.x / gj);
      e = make_float2(0.5f * (1.0f - gj), 0.0f);
    } else if (near) {
      e = make_float2(-0.5f * g.x, -0.5f * g.y);
    } else {
      const float rd = 1.0f / d;
      e = make_float2(c.x * rd, c.y * rd);
      l2 = fmaf(c.x * c.x + c.y * c.y, rd, l2);
    }
    emax = fmaxf(emax, fabsf(e.x) + fabsf(e.y));
#pragma unroll
    for (int m = 0; m < 32; ++m)
      if (m < n) cfma(xp[m], X[m * 32 + i], e);
  }
  __syncwarp();  // every lane is done reading the FP32 solve
  // One step leaves the square of the FP32 solve's error: a matrix whose correction exceeds
  // 2^-12 somewhere (an unusually poor FP32 eigenvector) is listed for a second step, which the
  // launcher runs on the listed matrices from this step's output; one that still needs it then
  // is flagged (WBG_FLAG_REFINE_WIDE).
  if (__any_sync(0xffffffffu, lane < n && emax > 0x1p-12f) && lane == 0 && valid) {
    if (relist) relist[1 + atomicAdd(relist, 1)] = (int)k;
    else atomicOr(errflag, WBG_FLAG_REFINE_WIDE);
  }
  if (inc) {     // a cluster's columns take x'_j (rounded) for the Rayleigh-Ritz step
#pragma unroll
    for (int m = 0; m < 32; ++m)
      if (m < n) {
        const float2 v = X[m * 32 + lane];
        X[m * 32 + lane] = make_float2(v.x + xp[m].x, v.y + xp[m].y);
      }
  }
  if (lane < n) lamd[lane] = lnew + (double)l2;
  __syncwarp();
  // column j = x + c (c: the correction, zero for a cluster's columns), normalised: |x + c|^2 with
  // |x|^2 in double-float and the small terms in FP32, s = 1 / |x + c| - 1, and each element
  // x + (c + (x + c) s) rounded once.  Columns outside clusters are written before the
  // Rayleigh-Ritz steps (their corrections need no registers past this point), the others after.
  auto write_column = [&](const bool with_corr) {
    df64 nr = df_from_f(0.0f);
    float small = 0.0f;
#pragma unroll
    for (int q = 0; q < 32; ++q)
      if (q < n) {
        const float2 v = X[q * 32 + j], cq = with_corr ? xp[q] : make_float2(0.0f, 0.0f);
        lz_fma_mixed(nr, df_from_f(v.x), v.x);
        lz_fma_mixed(nr, df_from_f(v.y), v.y);
        small = fmaf(2.0f * v.x + cq.x, cq.x, fmaf(2.0f * v.y + cq.y, cq.y, small));
      }
    const float sc = (float)(1.0 / sqrt(df_to_double(df_lazy_done(nr)) + (double)small) - 1.0);
    if (valid && lane < n) {
#pragma unroll
      for (int q = 0; q < 32; ++q)
        if (q < n) {
          const float2 v = X[q * 32 + lane], cq = with_corr ? xp[q] : make_float2(0.0f, 0.0f);
          const float tx = cq.x + (v.x + cq.x) * sc, ty = cq.y + (v.y + cq.y) * sc;
          U[k * strideU + q * n + lane] = make_float2(v.x + tx, v.y + ty);
        }
      E[k * n + lane] = lamd[lane];
    }
  };
  if (!inc) write_column(true);
  // Rayleigh-Ritz in each cluster: lane q holds row q of H X_c; sums over rows by shuffles
  for (int c0 = 0; c0 < n;) {
    int cend = c0 + 1;  // end of the cluster
    while (cend < n && !cstart[cend]) ++cend;
    const int c1 = min(cend, c0 + RF_MAXC);  // a wider cluster in runs of RF_MAXC
    if (cend - c0 > RF_MAXC && lane == 0 && valid) atomicOr(errflag, WBG_FLAG_REFINE_WIDE);
    const int m = c1 - c0;
    if (m > 1) {
      const int q = lane < n ? lane : n - 1;
      const bool row = lane < n;
      for (int t = 0; t < m; ++t) {
        df64 yr = df_from_f(0.0f), yi = df_from_f(0.0f);  // (H x'_t)_q
        for (int s = 0; s < n; ++s) lz_cfma_mixed(yr, yi, hs_elem(Hs, q, s), X[s * 32 + c0 + t]);
        const double2 y = make_double2(df_to_double(df_lazy_done(yr)), df_to_double(df_lazy_done(yi)));
        const float2 xt = X[q * 32 + c0 + t];
        for (int p = 0; p < m; ++p) {
          const float2 xf = X[q * 32 + c0 + p];
          const double2 xpq = make_double2(xf.x, xf.y);
          double2 pv = cmulc(xpq, y), gv = cmulc(xpq, make_double2(xt.x, xt.y));
          if (!row) pv = gv = make_double2(0.0, 0.0);
          pv.x = warp_sum(pv.x);
          pv.y = warp_sum(pv.y);
          gv.x = warp_sum(gv.x);
          gv.y = warp_sum(gv.y);
          if (lane == 0) {
            Pc[p * RF_MAXC + t] = pv;
            Gc[p * RF_MAXC + t] = gv;
          }
        }
      }
      __syncwarp();
      if (lane == 0) {  // Gc = L L^H, S = L^-H (over Gc); A = S^H P S = V mu V^H; W = S V (over P)
        double2 *S = Gc, *L = Ab, *Li = Vb;
        for (int j = 0; j < m; ++j) {  // Cholesky (the FP32 vectors of a cluster can be far from orthonormal)
          double dj = Gc[j * RF_MAXC + j].x;
          for (int t = 0; t < j; ++t) dj -= L[j * m + t].x * L[j * m + t].x + L[j * m + t].y * L[j * m + t].y;
          dj = sqrt(fmax(dj, 1e-30));
          L[j * m + j] = make_double2(dj, 0.0);
          for (int i = j + 1; i < m; ++i) {
            double2 t2 = Gc[i * RF_MAXC + j];
            for (int t = 0; t < j; ++t) t2 = csub(t2, cmul(L[i * m + t], cconj(L[j * m + t])));
            L[i * m + j] = make_double2(t2.x / dj, t2.y / dj);
          }
        }
        for (int j = 0; j < m; ++j) {  // L^-1, lower triangular
          for (int i = 0; i < j; ++i) Li[i * m + j] = make_double2(0.0, 0.0);
          Li[j * m + j] = make_double2(1.0 / L[j * m + j].x, 0.0);
          for (int i = j + 1; i < m; ++i) {
            double2 t2 = make_double2(0.0, 0.0);
            for (int t = j; t < i; ++t) t2 = cadd(t2, cmul(L[i * m + t], Li[t * m + j]));
            Li[i * m + j] = make_double2(-t2.x / L[i * m + i].x, -t2.y / L[i * m + i].x);
          }
        }
        for (int a = 0; a < m; ++a)
          for (int b = 0; b < m; ++b) S[a * RF_MAXC + b] = cconj(Li[b * m + a]);
        for (int a = 0; a < m; ++a)  // V <- P S
          for (int b = 0; b < m; ++b) {
            double2 t = make_double2(0.0, 0.0);
            for (int s = 0; s < m; ++s) t = cadd(t, cmul(Pc[a * RF_MAXC + s], S[s * RF_MAXC + b]));
            Vb[a * m + b] = t;
          }
        for (int a = 0; a < m; ++a)  // A <- S^H (P S)
          for (int b = 0; b < m; ++b) {
            double2 t = make_double2(0.0, 0.0);
            for (int s = 0; s < m; ++s) t = cadd(t, cmulc(S[s * RF_MAXC + a], Vb[s * m + b]));
            Ab[a * m + b] = t;
          }
        for (int a = 0; a < m; ++a)  // Hermitian part
          for (int b = a; b < m; ++b) {
            const double2 u = Ab[a * m + b], v = Ab[b * m + a];
            Ab[a * m + b] = make_double2(0.5 * (u.x + v.x), 0.5 * (u.y - v.y));
            Ab[b * m + a] = cconj(Ab[a * m + b]);
          }
        jacobi_herm(Ab, Vb, m);
        for (int a = 0; a < m; ++a) {
          lamd[c0 + a] = Ab[a * m + a].x;
          for (int b = 0; b < m; ++b) {
            double2 t = make_double2(0.0, 0.0);
            for (int s = 0; s < m; ++s) t = cadd(t, cmul(S[a * RF_MAXC + s], Vb[s * m + b]));
            Pc[a * RF_MAXC + b] = t;
          }
        }
      }
      __syncwarp();
      if (row) {  // row q of X_c <- X_c W, in FP64 from the FP32 values
        double2 xr[RF_MAXC];
#pragma unroll
        for (int b = 0; b < RF_MAXC; ++b) {
          xr[b] = make_double2(0.0, 0.0);
          if (b < m)
            for (int t = 0; t < m; ++t) {
              const float2 v = X[q * 32 + c0 + t];
              xr[b] = cadd(xr[b], cmul(make_double2(v.x, v.y), Pc[t * RF_MAXC + b]));
            }
        }
#pragma unroll
        for (int b = 0; b < RF_MAXC; ++b)
          if (b < m) X[q * 32 + c0 + b] = make_float2((float)xr[b].x, (float)xr[b].y);
      }
      __syncwarp();
    }
    c0 = c1;
  }
  if (inc) write_column(false);
}

// Shared memory of one SM (228 KB, 1 KB of it reserved per resident block) and the largest
// dynamic allocation this file asks of one block.
constexpr size_t kSmemPerSM = 228 * 1024, kSmemPerBlockReserved = 1024, kMaxBlockSmem = 220 * 1024;

// Matrices per block for a kernel whose groups take `smem` bytes of shared memory and
// `threads` threads each: the power of two up to gmax that keeps the most matrices resident
// on one SM (shared memory, 2048 threads and 32 blocks per SM); 0 if one group does not fit.
int pick_group(size_t smem, int threads, int gmax) {
  int best = 0, bestres = 0;
  for (int g = 1; g <= (gmax < 1 ? 1 : gmax); g *= 2) {
    const size_t blk = (size_t)g * smem;
    if (blk > kMaxBlockSmem) break;
    int bps = (int)(kSmemPerSM / (blk + kSmemPerBlockReserved));
    if (bps > 2048 / (g * threads)) bps = 2048 / (g * threads);
    if (bps > 32) bps = 32;
    if (bps * g >= bestres) { bestres = bps * g; best = g; }
  }
  return best;
}

// Launch shapes of the three kernels for n x n matrices (R: arithmetic of the solve, TU: type of
// the back-transform): lanes and shared memory per matrix, the largest group each kernel takes,
// the built-in choices, and which other group sizes fit (the autotuner's candidates).
template <typename R, typename TU>
struct EighShape {
  int L, LT, CW, gmaxT, gmaxV;
  size_t smT, smQ1, smV;  // shared memory per matrix: tridiagonalisation, QL (d and e), vectors
  explicit EighShape(int n) {
    typedef typename C2<R>::t CR;
    typedef typename C2<TU>::t VU;
    L = lanes_for(n);
    // tridiagonalisation: mirrored row pairs on half the lanes (balanced rows; one row per lane
    // on all 32 lanes measured 22% slower at nw = 32)
    LT = L >= 8 ? L / 2 : 4;
    gmaxT = 128 / LT;
    smT = ((size_t)n * (n + 1) / 2 + 2 * n) * sizeof(CR);
    smQ1 = 2 * (size_t)n * sizeof(R);  // d and e of one matrix (one thread per matrix)
    const size_t zbytes = (((size_t)n * n + 3 * n) * sizeof(R) + 15) / 16 * 16;
    const size_t vbytes = ((size_t)n * sizeof(VU) + 15) / 16 * 16;
    CW = n;  // back-transform chunk width: the whole U unless it does not fit next to Z
    auto ub = [&](int cw) { return kUOverlaysZ<R, TU> ? (size_t)0 : ((size_t)n * cw * sizeof(VU) + 15) / 16 * 16; };
    if (kUWideOverlay<R, TU> && (zbytes > ub(n) ? zbytes : ub(n)) + vbytes <= kMaxBlockSmem) {
      smV = (zbytes > ub(n) ? zbytes : ub(n)) + vbytes;  // U over Z (CW = n)
    } else {
      if (!kUOverlaysZ<R, TU> && zbytes + ub(n) + vbytes > kMaxBlockSmem) CW = 32;
      smV = zbytes + ub(CW) + vbytes;
    }
    gmaxV = 64 / L;
  }
  int tridiag_default() const { return pick_group(smT, LT, gmaxT); }
  int ql_default() const {
    int BQ = 128;  // threads (matrices) per block
    while (BQ > 32 && (size_t)BQ * smQ1 > 64 * 1024) BQ /= 2;
    return BQ;
  }
  int vectors_default() const { return pick_group(smV, L, gmaxV); }
  // a group size fits: power of two up to gmax whose shared memory fits one block, and whole
  // warps unless it is the largest size that fits (the heuristic's choice when memory-bound)
  static bool group_fits(int g, size_t smem, int lanes, int gmax) {
    if (g < 1 || g > gmax || (g & (g - 1)) || (size_t)g * smem > kMaxBlockSmem) return false;
    const bool larger = 2 * g <= gmax && (size_t)2 * g * smem <= kMaxBlockSmem;
    return (g * lanes) % 32 == 0 || !larger;
  }
  bool fits(int param, int v) const {
    if (param == WBG_TUNE_EIGH_TRIDIAG_GROUP) return group_fits(v, smT, LT, gmaxT);
    if (param == WBG_TUNE_EIGH_VECTORS_GROUP) return group_fits(v, smV, L, gmaxV);
    if (param == WBG_TUNE_EIGH_QL_BLOCK)
      return v >= 32 && v <= 256 && !(v & (v - 1)) && (size_t)v * smQ1 <= kMaxBlockSmem;
    return false;
  }
  // the tuned value of `param` when one is set and fits, else the built-in choice
  int choose(int param, int variant, int n, int dflt) const {
    const int t = wbg_tuned(param, variant, n);
    return (t > 0 && fits(param, t)) ? t : dflt;
  }
  int candidates(int param, int* values, int capacity) const {
    int count = 0;
    for (int v = 1; v <= 256; v *= 2)
      if (fits(param, v) && count < capacity) values[count++] = v;
    return count;
  }
};

template <typename R, typename TU, typename HIn, typename VO = typename C2<TU>::t>
int launch_eigh(const void* H, long long strideH, int n, int nk, void* E, void* U, long long strideU, int lowerIn,
                int valuesOnly, int stage, int variant, void* workspace, int* errflag, cudaStream_t stream) {
  typedef typename C2<R>::t CR;
  typedef typename C2<TU>::t VU;
  char* w = (char*)workspace;
  VU* Vh = (VU*)w; w += (size_t)nk * n * n * 16;
  VU* tau = (VU*)w; w += (size_t)nk * n * 16;
  R* d = (R*)w; w += (size_t)nk * n * 8;
  R* e = (R*)w;
  const EighShape<R, TU> sh(n);
  const int L = sh.L, LT = sh.LT;
  if (stage != 2) {  // stage 1 (or both): the tridiagonalisation into the workspace
    const size_t smT = sh.smT;
    const int G0 = sh.tridiag_default();
    if (G0 == 0) return WBG_ERR_SIZE;
    const int G = sh.choose(WBG_TUNE_EIGH_TRIDIAG_GROUP, variant, n, G0);
    cudaFuncSetAttribute(eigh_tridiag<R, HIn, TU>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxBlockSmem);
    eigh_tridiag<R, HIn, TU><<<(nk + G - 1) / G, G * LT, G * smT, stream>>>((const HIn*)H, strideH, n, nk, LT, G,
                                                                             lowerIn, Vh, tau, d, e);
    if (stage == 1) return wbg_cuda_status(cudaGetLastError());
  }
  const int BQ = sh.choose(WBG_TUNE_EIGH_QL_BLOCK, variant, n, sh.ql_default());
  const size_t smQ = (size_t)BQ * sh.smQ1;
  cudaFuncSetAttribute(eigh_ql<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxBlockSmem);
  eigh_ql<R><<<(nk + BQ - 1) / BQ, BQ, smQ, stream>>>(d, e, n, nk, (double*)E, errflag);
  if (valuesOnly) return wbg_cuda_status(cudaGetLastError());
  const int CW = sh.CW;
  const size_t smV = sh.smV;
  const int GV0 = sh.vectors_default();
  if (GV0 == 0) return WBG_ERR_SIZE;
  const int GV = sh.choose(WBG_TUNE_EIGH_VECTORS_GROUP, variant, n, GV0);
  cudaFuncSetAttribute(eigh_vectors<R, TU, VO>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxBlockSmem);
  eigh_vectors<R, TU, VO><<<(nk + GV - 1) / GV, GV * L, GV * smV, stream>>>(Vh, tau, d, e, (const double*)E, n, nk, L,
                                                                            GV, CW, (VO*)U, strideU);
  return wbg_cuda_status(cudaGetLastError());
}

// FP32 solve (tridiagonalisation, QL, inverse iteration, back-transform all in FP32) and one
// refinement step against the double-float or FP64 H (section 4)
template <typename HIn>
int launch_eigh_refined(const void* H, long long strideH, int n, int nk, void* E, void* U, long long strideU,
                        int lowerIn, int stage, void* workspace, int* errflag, cudaStream_t stream) {
  const int st = launch_eigh<float, float, HIn, float2>(H, strideH, n, nk, E, U, strideU, lowerIn, 0, stage, 5,
                                                       workspace, errflag, stream);
  if (st != WBG_OK || stage == 1) return st;
  const int G = 2;
  const size_t sm = G * RF_GROUP_BYTES;
  // list of the matrices that take a second step: [count, k ...] over the reflectors' workspace
  // (free once the back-transform has run)
  int* list = (int*)workspace;
  cudaMemsetAsync(list, 0, sizeof(int), stream);
  cudaFuncSetAttribute(eigh_refine<HIn>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  const unsigned grid = (unsigned)((nk + G - 1) / G);
  eigh_refine<HIn><<<grid, 32 * G, sm, stream>>>((const HIn*)H, strideH, n, nk, lowerIn, (float2*)U, strideU,
                                                (double*)E, G, errflag, nullptr, list);
  eigh_refine<HIn><<<grid, 32 * G, sm, stream>>>((const HIn*)H, strideH, n, nk, lowerIn, (float2*)U, strideU,
                                                (double*)E, G, errflag, list, nullptr);
  return wbg_cuda_status(cudaGetLastError());
}

}  // namespace

size_t wbg_eigh_workspace_bytes(int n, int nk) {
  // Vh (n*n complex) + tau (n complex) + d, e (n real each) per matrix; 8-byte reals in both modes
  return (size_t)nk * ((size_t)n * n * 16 + (size_t)n * 16 + 2 * (size_t)n * 8) + 1024;
}

int wbg_eigh_run(const void* H, long long strideH, int n, int nk, void* E, void* U, long long strideU, int mode,
                 void* workspace, size_t workspace_bytes, int* errflag, cudaStream_t stream) {
  const int vo = (mode & WBG_EIGH_VALUES) ? 1 : 0;
  const int stage = (mode & WBG_EIGH_STAGE1) ? 1 : (mode & WBG_EIGH_STAGE2) ? 2 : 0;
  if (n < 1 || n > WBG_EIGH_NMAX || nk < 1 || !E || (!U && !vo) || !errflag) return WBG_ERR_ARG;
  if (!H && stage != 2) return WBG_ERR_ARG;
  if (mode < 0 ||
      mode > (3 | WBG_EIGH_LOWER | WBG_EIGH_VALUES | WBG_EIGH_STAGE1 | WBG_EIGH_STAGE2 | WBG_EIGH_PRECISE_VECTORS |
              WBG_EIGH_DF64_VECTORS | WBG_EIGH_REFINE))
    return WBG_ERR_ARG;
  if (mode & WBG_EIGH_REFINE) {  // FP32 solve + refinement: modes 2 / 3, eigenvectors, n <= 32
    if ((mode & 3) < 2 || n > 32 || vo || (mode & (WBG_EIGH_PRECISE_VECTORS | WBG_EIGH_DF64_VECTORS)) || !H ||
        ((mode & WBG_EIGH_STAGE1) && (mode & WBG_EIGH_STAGE2)))
      return WBG_ERR_ARG;
    if (workspace_bytes < wbg_eigh_workspace_bytes(n, nk)) return WBG_ERR_WORKSPACE;
    const int lo = (mode & WBG_EIGH_LOWER) ? 1 : 0;
    if ((mode & 3) == 2)
      return launch_eigh_refined<double2>(H, strideH, n, nk, E, U, strideU, lo, stage, workspace, errflag, stream);
    return launch_eigh_refined<cdf>(H, strideH, n, nk, E, U, strideU, lo, stage, workspace, errflag, stream);
  }
  if ((mode & WBG_EIGH_DF64_VECTORS) && (!(mode & WBG_EIGH_PRECISE_VECTORS) || (mode & 3) < 2)) return WBG_ERR_ARG;
  if ((mode & WBG_EIGH_STAGE1) && (mode & WBG_EIGH_STAGE2)) return WBG_ERR_ARG;
  if (workspace_bytes < wbg_eigh_workspace_bytes(n, nk)) return WBG_ERR_WORKSPACE;
  const int lo = (mode & WBG_EIGH_LOWER) ? 1 : 0;
  if ((mode & WBG_EIGH_PRECISE_VECTORS) && (mode & 3) != 1) {
    // back-transform (and its reflectors) in the solve's precision, U rounded to complex64 once,
    // or kept in double-float (WBG_EIGH_DF64_VECTORS)
    if ((mode & WBG_EIGH_DF64_VECTORS) && (mode & 3) == 2)
      return launch_eigh<df64, df64, double2, cdf>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 4, workspace,
                                                    errflag, stream);
    if ((mode & WBG_EIGH_DF64_VECTORS) && (mode & 3) == 3)
      return launch_eigh<df64, df64, cdf, cdf>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 4, workspace,
                                                errflag, stream);
    switch (mode & 3) {
      case 0:
        return launch_eigh<double, double, double2, float2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 1,
                                                             workspace, errflag, stream);
      case 2:
        return launch_eigh<df64, df64, double2, float2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 4,
                                                         workspace, errflag, stream);
      default:
        return launch_eigh<df64, df64, cdf, float2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 4, workspace,
                                                     errflag, stream);
    }
  }
  switch (mode & 3) {
    case 1:
      return launch_eigh<double, double, double2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 1, workspace,
                                                  errflag, stream);
    case 0:
      return launch_eigh<double, float, double2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 0, workspace,
                                                 errflag, stream);
    case 2:
      return launch_eigh<df64, float, double2>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 2, workspace,
                                               errflag, stream);
    default:
      return launch_eigh<df64, float, cdf>(H, strideH, n, nk, E, U, strideU, lo, vo, stage, 3, workspace, errflag,
                                           stream);
  }
}

int wbg_eigh_tune_candidates(int param, int n, int variant, int* values, int capacity) {
  if (n < 1 || n > WBG_EIGH_NMAX) return 0;
  switch (variant) {  // eigh mode & 3 (4: double-float solve and back-transform): the (solve, back-transform) types
    case 1: return EighShape<double, double>(n).candidates(param, values, capacity);
    case 0: return EighShape<double, float>(n).candidates(param, values, capacity);
    case 4: return EighShape<df64, df64>(n).candidates(param, values, capacity);
    case 5: return EighShape<float, float>(n).candidates(param, values, capacity);
    default: return EighShape<df64, float>(n).candidates(param, values, capacity);
  }
}

// ---------------------------------------------------------------------------------------
// Allocation-free variant of wbg_eigh_batched.
//
// Some callers cannot call cudaMalloc: a plugin inside a host application whose memory
// manager owns all of the GPU's memory (a framework's caching allocator, an embedding
// application with a fixed budget), a real-time loop that forbids allocation after start-up
// because cudaMalloc / cudaFree may synchronise the device and take unbounded time, and a
// thin FFI binding (ctypes, cgo) that has no device allocator of its own.  For them the
// eigensolver's workspace lives in a fixed file-scope device array instead of a caller- or
// library-allocated buffer.  The array is part of the module: every GPU that loads this
// library holds WBG_EIGH_NOALLOC_SCRATCH_BYTES of it until the process exits.  All calls
// share it, so calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race and must be serialised by the caller.  Every workspace word is
// written by the kernels before it is read, so the contents left by a previous call never
// need clearing.  The two-call split (WBG_EIGH_STAGE1 / STAGE2) is refused here: any other
// call between the two stages would overwrite the tridiagonal factors in the shared array.
// ---------------------------------------------------------------------------------------
#include <mutex>
#include <cuda.h>

static __device__ __align__(256) unsigned char g_eigh_noalloc_scratch[WBG_EIGH_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
struct NoallocSlot {
  void* ptr = nullptr;
  unsigned long long ctx_id = 0;  // context whose module the address belongs to
};
NoallocSlot g_noalloc[kMaxDevices];
std::mutex g_noalloc_mutex;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// Unique id of the current context (cuCtxGetId through the runtime's driver entry points, so
// the library needs no link-time dependency on libcuda); 0 when the driver cannot say.
unsigned long long current_context_id() {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)f;
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS) return id;
  return 0;
}

// Device address of the scratch array in the current context.  In host code the array's name
// is only a host-side stand-in, so the address is looked up with cudaGetSymbolAddress (with
// the device current) on the first call on each device and cached with the id of the context
// it belongs to.  A context torn down and recreated (cudaDeviceReset, a released primary
// context) reloads the module, and the array may then sit elsewhere: a call that finds a new
// context id looks the address up again.
int noalloc_scratch(void** ptr) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return WBG_ERR_CUDA;
  const unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoallocSlot& slot = g_noalloc[dev];
  if (!slot.ptr || id == 0 || slot.ctx_id != id) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_eigh_noalloc_scratch) != cudaSuccess || !p) return WBG_ERR_CUDA;
    slot.ptr = p;
    slot.ctx_id = id;
  }
  *ptr = slot.ptr;
  return WBG_OK;
}
}  // namespace

extern "C" int wbg_eigh_batched_noalloc(const void* H, long long strideH, int nw, int nk, double* E, void* U,
                                        long long strideU, int mode, int* errflag, void* stream) {
  // the argument rules of wbg_eigh_batched (U may be NULL for eigenvalues only), without the
  // two-stage split, whose tridiagonal factors could not survive another call in between
  if (mode & (WBG_EIGH_STAGE1 | WBG_EIGH_STAGE2)) return WBG_ERR_ARG;
  if (nw < 1 || nw > WBG_EIGH_NMAX || nk < 1 || !H || !E || (!U && !(mode & WBG_EIGH_VALUES)) || !errflag)
    return WBG_ERR_ARG;
  const size_t need = wbg_eigh_workspace_bytes(nw, nk);
  if (need > (size_t)WBG_EIGH_NOALLOC_SCRATCH_BYTES) return WBG_ERR_SIZE;  // batch too large for the scratch
  void* ws = nullptr;
  const int st = noalloc_scratch(&ws);
  if (st != WBG_OK) return st;
  return wbg_eigh_run(H, strideH, nw, nk, E, U, strideU, mode, ws, need, errflag, (cudaStream_t)stream);
}
