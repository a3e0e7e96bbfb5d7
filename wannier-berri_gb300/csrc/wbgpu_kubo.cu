// Dynamic (Kubo-type) calculators (stage 4).
//
// Replaces calculators/dynamic.py:26-360: DynamicCalculator.__call__ (:71-114) with the
// formulas and frequency factors of OpticalConductivity (:170-196), JDOS (:133-162), SHC
// (:199-236, spin current of formula/covariant.py:689-756), ShiftCurrent (:239-316) and
// InjectionCurrent (:319-360):
//   restot[E_F][w][c] += sum_{group pairs (G1, G2)} f_w(E1, E2) f_E(E1, E2) M^c(G1, G2)
//   M^c = sum_{n in G1, m in G2} I^c_nm (the formula's trace_ln),  f_E = FD(E2) - FD(E1).
// Element tensors (D_nm = -V_nm / (E_n - E_m), A = i D + Abar, data_K.py:290-334):
//   optical conductivity  i A^a_nm A^b_mn                                   9 complex, (a, b)
//   JDOS                  1                                                 1 real
//   SHC                   Im(J^{as}_nm (-i A^b_mn))                         27 real, (a, b, s)
//   shift current         -Im(dA^{ca}_nm A^b_mn) + (b <-> c)                27 real, (a, b, c)
//   injection current     (v^a_n - v^a_m) A^b_nm A^c_mn                     27 complex, (a, b, c)
// with J the spin-current matrix (simple / qiao / ryoo) and dA the generalised derivative of
// A with principal-value D (broadening sc_eta).
// kubo_pairs:  one CTA per k-point: groups over all bands (degen_thresh), one thread per
//              ordered pair of groups kept by `nonzero` (dynamic.py:65-69; JDOS :158-162); the
//              element tensors are computed in place from the band-basis fields, with sums over
//              the intermediate bands for SHC and the shift current.  One record per pair:
//              E2 - E1 (FP64), f_E per level and M (FP32 in the mixed path, FP64 in the
//              FP64 path).
// kubo_accum:  one thread per frequency, a chunk of levels per block (grid z), a chunk of
//              k-points per block (grid y): accumulation in shared memory in the records'
//              precision, fixed-point sums into the result (FP64 path, and JDOS).
// kubo_gemm:   the mixed path's 9- and 27-component sums as a register-tiled complex GEMM
//              (frequencies x (level, component) per k-point, records as the contraction).
#include <float.h>
#include "wbgpu_common.cuh"
#include "wbgpu_fixed.cuh"
#include "wbgpu_kubo.cuh"
#include "wbgpu_spin.cuh"
#include "wbgpu_tune.cuh"

namespace {

__device__ double fermi_dirac(double E, double mu, double kBT) {
  if (kBT == 0.0) return E <= mu ? 1.0 : 0.0;
  if (mu > E + 30 * kBT) return 1.0;
  if (mu < E - 30 * kBT) return 0.0;
  return 1.0 / (exp((E - mu) / kBT) + 1.0);
}

// the three spin-current kinds share SHC's frequency factor
constexpr int kShcFactor = 100;

__host__ __device__ constexpr int dyn_ncomp(int f) {
  return f == WBG_DYN_OPTCOND ? 9 : f == WBG_DYN_JDOS ? 1 : 27;
}

// M += I_nm of formula F for the element (n, m), n in G1, m in G2
template <typename T, int F>
WBG_D void add_element(const KBand<T>& b, int n, int m, typename C2<T>::t* M) {
  typedef typename C2<T>::t V;
  if (F == WBG_DYN_JDOS) {
    M[0].x += T(1);
  } else if (F == WBG_DYN_OPTCOND) {
    V Anm[3], Amn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      Anm[a] = b.AH(a, n, m);
      Amn[a] = b.AH(a, m, n);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) M[3 * a + c] = cadd(M[3 * a + c], cmuli(cmul(Anm[a], Amn[c])));
  } else if (F == WBG_DYN_INJECTION) {
    V Anm[3], Amn[3];
    T dv[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      Anm[a] = b.AH(a, n, m);
      Amn[a] = b.AH(a, m, n);
      dv[a] = b.x(b.f.V + a, n, n).x - b.x(b.f.V + a, m, m).x;
    }
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const V t = cmul(Anm[bb], Amn[c]);
#pragma unroll
        for (int a = 0; a < 3; ++a) M[9 * a + 3 * bb + c] = cadd(M[9 * a + 3 * bb + c], cscale(t, dv[a]));
      }
  } else if (F == WBG_DYN_SHC_SIMPLE || F == WBG_DYN_SHC_QIAO || F == WBG_DYN_SHC_RYOO) {
    V J[9], Jt[9];
    spin_current<T, F>(b, n, m, J);
    spin_current<T, F>(b, m, n, Jt);
#pragma unroll
    for (int i = 0; i < 9; ++i) J[i] = cscale(cadd(J[i], cconj(Jt[i])), T(0.5));
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      const V A = b.AH(bb, m, n);
      const V B = mkc<T>(A.y, -A.x);  // -i A
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int s = 0; s < 3; ++s) M[9 * a + 3 * bb + s].x += cmul(J[3 * a + s], B).y;
    }
  } else {  // WBG_DYN_SHIFT
    // H[3c+a] = W + sum_HD + DV (times i / (E_m - E_n) below), X[3c+a] = the external terms
    V H[9], X[9];
    const bool ext = b.f.external_terms;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        H[3 * c + a] = b.x(b.f.W + 3 * c + a, n, m);
        X[3 * c + a] = ext ? b.x(b.f.dA + 3 * c + a, n, m) : czero<V>();
      }
    for (int l = 0; l < b.nw; ++l) {
      V Vnl[3], Vlm[3], Dlm[3], Dnl[3], Anl[3], Alm[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Vnl[a] = b.x(b.f.V + a, n, l);
        Vlm[a] = b.x(b.f.V + a, l, m);
        Dlm[a] = b.Dp(a, l, m);
        Dnl[a] = b.Dp(a, n, l);
        if (ext) {
          Anl[a] = b.x(b.f.A + a, n, l);
          Alm[a] = b.x(b.f.A + a, l, m);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          cfma(H[3 * c + a], Vnl[c], Dlm[a]);
          cfma(H[3 * c + a], cscale(Dnl[a], T(-1)), Vlm[c]);
          if (ext) {
            cfma(X[3 * c + a], Anl[c], Dlm[a]);
            cfma(X[3 * c + a], cscale(Dnl[a], T(-1)), Alm[c]);
          }
        }
    }
    V Vnn[3], Vmm[3], Dnm[3], Pnm[3], Ann[3], Amm[3], Anm[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      Vnn[a] = b.x(b.f.V + a, n, n);
      Vmm[a] = b.x(b.f.V + a, m, m);
      Dnm[a] = b.D(a, n, m);
      Pnm[a] = b.Dp(a, n, m);
      if (ext) {
        Ann[a] = b.x(b.f.A + a, n, n);
        Amm[a] = b.x(b.f.A + a, m, m);
        Anm[a] = b.x(b.f.A + a, n, m);
      }
    }
    const T dinv_mn = b.dinv(m, n);
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        V h = H[3 * c + a];
        // - V_nn^c Dp_nm^a + Dp_nm^a V_mm^c  and  DV: D^c_nm (V^a_nn - V^a_mm) + D^a_nm (V^c_nn - V^c_mm)
        h = cadd(h, cmul(Pnm[a], csub(Vmm[c], Vnn[c])));
        h = cadd(h, cmul(Dnm[c], csub(Vnn[a], Vmm[a])));
        h = cadd(h, cmul(Dnm[a], csub(Vnn[c], Vmm[c])));
        V g = cscale(cmuli(h), dinv_mn);
        if (ext) {
          V x = X[3 * c + a];
          x = cadd(x, cmul(Pnm[a], csub(Amm[c], Ann[c])));
          x = cadd(x, cmul(Dnm[c], csub(Ann[a], Amm[a])));
          x = cadd(x, cmul(Dnm[a], csub(Ann[c], Amm[c])));
          x = csub(x, cmuli(cmul(csub(Ann[a], Amm[a]), Anm[c])));
          g = cadd(g, x);
        }
        H[3 * c + a] = g;  // the generalised derivative dA^{c a}_nm
      }
    V Amn[3];
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) Amn[bb] = b.AH(bb, m, n);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int bb = 0; bb < 3; ++bb)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          M[9 * a + 3 * bb + c].x -= cmul(H[3 * c + a], Amn[bb]).y + cmul(H[3 * bb + a], Amn[c]).y;
  }
}

// grid: nk blocks of 128 threads.  Records of k-point k occupy slots [k*P, k*P + count[k]).
template <typename T, int F>
__global__ void kubo_pairs(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar,
                           wbg_dynamic_spec fs, int nw, WbgKubo kp, const double* __restrict__ efermi,
                           double* __restrict__ rec_dE, T* __restrict__ rec_fE, typename C2<T>::t* __restrict__ rec_M,
                           int* __restrict__ count, int P) {
  typedef typename C2<T>::t V;
  constexpr int NC = dyn_ncomp(F);
  extern __shared__ double smk[];
  double* Es = smk;                                   // [nw]
  double* Eg = Es + nw;                               // [nw] group mean energies
  int* gstart = reinterpret_cast<int*>(Eg + nw);      // [nw+1] group borders
  int* flag = gstart + nw + 1;                        // [nw]
  __shared__ int ng, cnt;
  const long long k = blockIdx.x;
  const long long nw2 = (long long)nw * nw;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) Es[i] = E[k * nw + i];
  __syncthreads();
  for (int i = threadIdx.x; i < nw; i += blockDim.x) flag[i] = (i == 0) || (Es[i] - Es[i - 1] > kp.degen_thresh);
  __syncthreads();
  if (threadIdx.x == 0) {
    int g = 0;
    for (int i = 0; i < nw; ++i)
      if (flag[i]) gstart[g++] = i;
    gstart[g] = nw;
    ng = g;
    cnt = 0;
  }
  __syncthreads();
  for (int g = threadIdx.x; g < ng; g += blockDim.x) {
    double s = 0.0;
    for (int i = gstart[g]; i < gstart[g + 1]; ++i) s += Es[i];
    Eg[g] = s / (double)(gstart[g + 1] - gstart[g]);
  }
  __syncthreads();
  KBand<T> band;
  band.X = Xbar ? Xbar + k * nFbar * nw2 : nullptr;
  band.E = Es;
  band.nw = nw;
  band.nw2 = nw2;
  band.f = fs;
  const double eocc1max = kp.EFmin - 30.0 * kp.kBT, eocc0min = kp.EFmax + 30.0 * kp.kBT;
  // Records are stored in pair order (slot = number of kept pairs before this one), so the
  // accumulation over them runs in the same order on every run: a block-wide exclusive count of
  // the kept pairs per round of blockDim.x pairs (warp ballots, warp totals in shared memory).
  __shared__ int warp_kept[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
  for (int base = 0; base < ng * ng; base += blockDim.x) {
    const int pr = base + threadIdx.x;
    const int g1 = pr < ng * ng ? pr / ng : 0, g2 = pr < ng * ng ? pr % ng : 0;
    bool keep = pr < ng * ng && g1 != g2;  // f_E(E, E) = 0
    const double E1 = Eg[g1], E2 = Eg[g2];
    if (keep) {
      if (F == WBG_DYN_JDOS) {
        const double d = E1 - E2;
        keep = E1 < kp.EFmax && E2 > kp.EFmin && fs.omega_min - 5 * kp.eta < d && d < fs.omega_max + 5 * kp.eta;
      } else {
        keep = !((E1 < eocc1max && E2 < eocc1max) || (E1 > eocc0min && E2 > eocc0min));
      }
    }
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_kept[wid] = __popc(ball);
    __syncthreads();
    int before = cnt;
    for (int w = 0; w < wid; ++w) before += warp_kept[w];
    const int slot = before + __popc(ball & ((1u << lane) - 1u));
    int total = 0;
    for (int w = 0; w < nwarps; ++w) total += warp_kept[w];
    __syncthreads();
    if (threadIdx.x == 0) cnt += total;  // read by the next round after its first barrier
    if (!keep) continue;
    V M[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) M[i] = czero<V>();
    for (int n = gstart[g1]; n < gstart[g1 + 1]; ++n)
      for (int m = gstart[g2]; m < gstart[g2 + 1]; ++m) add_element<T, F>(band, n, m, M);
    const long long r = k * (long long)P + slot;
    rec_dE[r] = E2 - E1;
    for (int e = 0; e < kp.nEF; ++e)
      rec_fE[r * kp.nEF + e] = (T)(fermi_dirac(E2, efermi[e], kp.kBT) - fermi_dirac(E1, efermi[e], kp.kBT));
#pragma unroll
    for (int i = 0; i < NC; ++i) rec_M[r * NC + i] = M[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) count[k] = cnt;
}

// smearing of dynamic.py:50-55 (utility.py:147-168), in the precision R of the accumulation
template <typename R>
__device__ R smear(R x, R eta, int gaussian) {
  if (gaussian) {
    const R y = x / eta;
    return fabs(x) < eta * R(14.142135623730951) ? R(0.5641895835477563) / eta * exp(-y * y) : R(0);
  }
  return R(0.3183098861837907) * eta / (x * x + eta * eta);
}

// f_w(E1, E2) from dE = E2 - E1 (FP64 difference with the frequency, precision R from there on:
// FP32 in the mixed path, FP64 in the FP64 path)
template <typename R>
__device__ typename C2<R>::t factor_omega(int formula, double dE, double om, R eta, int gaussian) {
  if (formula == WBG_DYN_OPTCOND || formula == kShcFactor) {
    // optical: (E2 - E1) / (E2 - E1 - w - i eta);  SHC: 1 / (E1 - E2 - w - i eta) / 2
    const bool opt = formula == WBG_DYN_OPTCOND;
    const R delta = (R)(opt ? dE - om : -dE - om);
    const R den = R(1) / (delta * delta + eta * eta);
    R cre = delta * den, cim = eta * den;
    if (gaussian) {
      const R x = delta / eta;
      cim = fabs(delta) < eta * R(14.142135623730951) ? R(1.7724538509055160) / eta * exp(-x * x) : R(0);
    }
    const R s = opt ? (R)dE : R(0.5);
    return mkc<R>(s * cre, s * cim);
  }
  R v = smear<R>((R)(-dE - om), eta, gaussian);  // JDOS, injection: smear(E1 - E2 - w)
  if (formula == WBG_DYN_SHIFT) v += smear<R>((R)(dE - om), eta, gaussian);
  return mkc<R>(v, R(0));
}

// grid: (ceil(nOmega / TPB), k chunks, level chunks); out: [nEF][nOmega][NC] complex entries, real
// and imaginary part each a fixed-point entry of wbgpu_fixed.cuh (order-independent sums over the
// blocks of k-points), then the count of non-finite contributions.  The block's sums of one
// k-point's pair records are added to `out` after that k-point, so an FP32 accumulation chain
// spans one k-point's records, not a chunk of k-points.
// R: precision of the records and the accumulation (float: mixed path, double: FP64 path)
template <int NC, typename R>
__global__ void kubo_accum(const double* __restrict__ rec_dE, const R* __restrict__ rec_fE,
                           const typename C2<R>::t* __restrict__ rec_M, const int* __restrict__ count, int P, int nk,
                           int kchunk, const double* __restrict__ omega, WbgKubo kp, int formula, int efc,
                           wbg_u64* __restrict__ out) {
  typedef typename C2<R>::t V;
  constexpr int nc = NC;
  extern __shared__ unsigned char smacc[];
  V* acc = reinterpret_cast<V*>(smacc);  // [efc][NC][blockDim.x]
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = w < kp.nOmega;
  const int e0 = blockIdx.z * efc;
  const int ne = min(efc, kp.nEF - e0);
  for (int i = 0; i < ne * nc; ++i) acc[i * blockDim.x + threadIdx.x] = czero<V>();
  const double om = active ? omega[w] : 0.0;
  const R eta = (R)kp.eta;
  const int fgroup = formula >= WBG_DYN_SHC_SIMPLE && formula <= WBG_DYN_SHC_RYOO ? kShcFactor : formula;
  const long long k0 = (long long)blockIdx.y * kchunk;
  const long long k1 = min((long long)nk, k0 + kchunk);
  wbg_u64* bad = out + 4 * (long long)kp.nEF * kp.nOmega * nc;
  for (long long k = k0; k < k1; ++k) {
    const int nrec = count[k];
    for (int q = 0; q < nrec; ++q) {
      const long long r = k * (long long)P + q;
      const V fw = factor_omega<R>(fgroup, rec_dE[r], om, eta, kp.gaussian);
      V Mv[NC];
#pragma unroll
      for (int i = 0; i < NC; ++i) Mv[i] = rec_M[r * NC + i];
      for (int e = 0; e < ne; ++e) {
        const R fe = rec_fE[r * kp.nEF + e0 + e];
        if (fe == R(0)) continue;
        const V c = mkc<R>(fe * fw.x, fe * fw.y);
#pragma unroll
        for (int i = 0; i < NC; ++i) {
          V& a = acc[(e * NC + i) * blockDim.x + threadIdx.x];
          a.x = fma(c.x, Mv[i].x, fma(-c.y, Mv[i].y, a.x));
          a.y = fma(c.x, Mv[i].y, fma(c.y, Mv[i].x, a.y));
        }
      }
    }
    if (nrec > 0 && active)
      for (int e = 0; e < ne; ++e)
        for (int i = 0; i < nc; ++i) {
          V& a = acc[(e * nc + i) * blockDim.x + threadIdx.x];
          wbg_u64* o = out + 4 * (((long long)(e0 + e) * kp.nOmega + w) * nc + i);
          fx_add_double(o, (double)a.x, bad);
          fx_add_double(o + 2, (double)a.y, bad);
          a = czero<V>();
        }
  }
}

// ---------------------------------------------------------------------------------------
// Mixed path, NC = 9 or 27: the same sums as a register-tiled complex GEMM per k-point,
//   out[w][(e, c)] += sum_r F[w][r] G[r][(e, c)],   F = f_w(dE_r), G = f_E[r][e] M[r][c]
// (calculators/dynamic.py:97-98: restot += factor_omega @ (factor_Efermi x M)).  A block takes
// a tile of KG_TW frequencies x KG_TC columns (e, c) and a chunk of k-points; per chunk of
// KG_RC records F and G are staged in shared memory (F from the FP64 difference dE - w, then
// FP32) and every thread accumulates a 4 x 8 tile of outputs in FP32 registers.  Sums run in
// three levels: a record chunk in FP32, the chunks of one k-point in FP32, the k-points of the
// block in FP64 (shared memory), so that no FP32 chain is longer than one k-point's chunks;
// the block's FP64 sums go to `out` once, as fixed-point entries.
// ---------------------------------------------------------------------------------------
constexpr int KG_TW = 64, KG_TC = 128, KG_RC = 32, KG_THR = 256;
constexpr size_t KG_SMEM = (size_t)32 * KG_THR * sizeof(double2) + (size_t)KG_RC * (KG_TW + KG_TC) * sizeof(float2);

template <int NC>
__global__ void __launch_bounds__(KG_THR, 1)
    kubo_gemm(const double* __restrict__ rec_dE, const float* __restrict__ rec_fE, const float2* __restrict__ rec_M,
              const int* __restrict__ count, int P, int nk, int kchunk, const double* __restrict__ omega, WbgKubo kp,
              int formula, wbg_u64* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smg[];
  double2* accd = reinterpret_cast<double2*>(smg);  // [32][KG_THR]: thread tid's output q at q * KG_THR + tid
  float2* Fs = reinterpret_cast<float2*>(accd + 32 * KG_THR);  // [KG_RC][KG_TW]
  float2* Gs = Fs + KG_RC * KG_TW;                             // [KG_RC][KG_TC]
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int w0 = blockIdx.x * KG_TW, col0 = blockIdx.z * KG_TC;
  const int ncol = kp.nEF * NC;
  const float eta = (float)kp.eta;
  const int fgroup = formula >= WBG_DYN_SHC_SIMPLE && formula <= WBG_DYN_SHC_RYOO ? kShcFactor : formula;
  for (int q = 0; q < 32; ++q) accd[q * KG_THR + tid] = make_double2(0.0, 0.0);
  const long long k0 = (long long)blockIdx.y * kchunk;
  const long long k1 = min((long long)nk, k0 + kchunk);
  for (long long k = k0; k < k1; ++k) {
    const int nrec = count[k];
    if (nrec == 0) continue;
    const long long rbase = k * (long long)P;
    float2 acck[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acck[i][j] = make_float2(0.f, 0.f);
    for (int r0 = 0; r0 < nrec; r0 += KG_RC) {
      const int rn = min(KG_RC, nrec - r0);
      // the chunk's loads all issued before any is used (one memory latency per chunk)
      constexpr int PF = KG_RC * KG_TW / KG_THR, PG = KG_RC * KG_TC / KG_THR;
      double dEv[PF], omv[PF];
      float fev[PG];
      float2 mv[PG];
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int idx = q * KG_THR + tid, r = idx / KG_TW, w = idx % KG_TW;
        const bool ok = r < rn && w0 + w < kp.nOmega;
        dEv[q] = ok ? __ldg(rec_dE + rbase + r0 + r) : 0.0;
        omv[q] = ok ? __ldg(omega + w0 + w) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < PG; ++q) {
        const int idx = q * KG_THR + tid, r = idx / KG_TC, col = col0 + idx % KG_TC;
        const bool ok = r < rn && col < ncol;
        const int e = col / NC, c = col - e * NC;
        const long long rr = rbase + r0 + r;
        fev[q] = ok ? __ldg(rec_fE + rr * kp.nEF + e) : 0.f;
        mv[q] = ok ? __ldg(rec_M + rr * NC + c) : make_float2(0.f, 0.f);
      }
      __syncthreads();  // the previous chunk's tiles are read
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int idx = q * KG_THR + tid, r = idx / KG_TW, w = idx % KG_TW;
        Fs[idx] = (r < rn && w0 + w < kp.nOmega) ? factor_omega<float>(fgroup, dEv[q], omv[q], eta, kp.gaussian)
                                                 : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int q = 0; q < PG; ++q) Gs[q * KG_THR + tid] = make_float2(fev[q] * mv[q].x, fev[q] * mv[q].y);
      __syncthreads();
      float2 acc[4][8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int r = 0; r < KG_RC; ++r) {
        float2 f[4], g[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) f[i] = Fs[r * KG_TW + ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 8; ++j) g[j] = Gs[r * KG_TC + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            acc[i][j].x = fmaf(f[i].x, g[j].x, fmaf(-f[i].y, g[j].y, acc[i][j].x));
            acc[i][j].y = fmaf(f[i].x, g[j].y, fmaf(f[i].y, g[j].x, acc[i][j].y));
          }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          acck[i][j].x += acc[i][j].x;
          acck[i][j].y += acc[i][j].y;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        double2& a = accd[(i * 8 + j) * KG_THR + tid];
        a.x += (double)acck[i][j].x;
        a.y += (double)acck[i][j].y;
      }
  }
  wbg_u64* bad = out + 4 * (long long)kp.nEF * kp.nOmega * NC;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int w = w0 + ty + 16 * i, col = col0 + tx + 16 * j;
      if (w >= kp.nOmega || col >= ncol) continue;
      const int e = col / NC, c = col - e * NC;
      const double2 a = accd[(i * 8 + j) * KG_THR + tid];
      wbg_u64* o = out + 4 * (((long long)e * kp.nOmega + w) * NC + c);
      fx_add_double(o, a.x, bad);
      fx_add_double(o + 2, a.y, bad);
    }
}

template <typename T>
void launch_pairs(int formula, int nk, size_t smp, cudaStream_t stream, const double* E, const void* Xbar, int nFbar,
                  const wbg_dynamic_spec& fs, int nw, const WbgKubo& kp, const double* efermi, double* rec_dE,
                  void* rec_fE, void* rec_M, int* count, int P) {
  typedef typename C2<T>::t V;
  const V* X = (const V*)Xbar;
#define WBG_PAIRS(F) kubo_pairs<T, F><<<nk, 128, smp, stream>>>(E, X, nFbar, fs, nw, kp, efermi, rec_dE, (T*)rec_fE, \
                                                                (V*)rec_M, count, P)
  switch (formula) {
    case WBG_DYN_OPTCOND: WBG_PAIRS(WBG_DYN_OPTCOND); break;
    case WBG_DYN_JDOS: WBG_PAIRS(WBG_DYN_JDOS); break;
    case WBG_DYN_SHC_SIMPLE: WBG_PAIRS(WBG_DYN_SHC_SIMPLE); break;
    case WBG_DYN_SHC_QIAO: WBG_PAIRS(WBG_DYN_SHC_QIAO); break;
    case WBG_DYN_SHC_RYOO: WBG_PAIRS(WBG_DYN_SHC_RYOO); break;
    case WBG_DYN_SHIFT: WBG_PAIRS(WBG_DYN_SHIFT); break;
    default: WBG_PAIRS(WBG_DYN_INJECTION); break;
  }
#undef WBG_PAIRS
}

bool field_ok(int first, int n, int nFbar) { return first >= 0 && first + n <= nFbar; }

}  // namespace

int wbg_dynamic_ncomp_impl(int formula) {
  return formula >= WBG_DYN_OPTCOND && formula <= WBG_DYN_INJECTION ? dyn_ncomp(formula) : 0;
}

// Records per pair slot: E2 - E1 (double), f_E per level and M (complex), both sized for the
// FP64 path (the mixed path stores them in FP32 in the first half of each region).
size_t wbg_dynamic_workspace_bytes(int formula, int nw, int nk, int nEF) {
  const size_t P = (size_t)nw * nw;
  const size_t nc = (size_t)wbg_dynamic_ncomp_impl(formula);
  return (size_t)nk * P * (8 + 8 * (size_t)nEF + 16 * nc) + (size_t)nk * 4 + 1024;
}

int wbg_dynamic_run(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* fs, int nw, int nk,
                    const WbgKubo* kp, const double* efermi, const double* omega, void* workspace,
                    size_t workspace_bytes, void* out, int fp64, cudaStream_t stream) {
  if (!E || !fs || !kp || !efermi || !omega || !workspace || !out || nw < 1 || nk < 1) return WBG_ERR_ARG;
  const int F = fs->formula;
  const int nc = wbg_dynamic_ncomp_impl(F);
  if (nc == 0 || (fp64 != 0 && fp64 != 1)) return WBG_ERR_ARG;
  if (kp->nEF < 1 || kp->nEF > 4096 || kp->nOmega < 1 || !(kp->eta > 0.0)) return WBG_ERR_ARG;
  const int ext = fs->external_terms;
  if (ext != 0 && ext != 1) return WBG_ERR_ARG;
  if (F != WBG_DYN_JDOS) {  // fields each formula reads
    if (!Xbar || !field_ok(fs->V, 3, nFbar)) return WBG_ERR_ARG;
    const bool needA = ext || F == WBG_DYN_SHC_QIAO || F == WBG_DYN_SHC_RYOO;
    if ((F == WBG_DYN_SHC_QIAO || F == WBG_DYN_SHC_RYOO) && !ext) return WBG_ERR_ARG;
    if (needA && !field_ok(fs->A, 3, nFbar)) return WBG_ERR_ARG;
    if (F >= WBG_DYN_SHC_SIMPLE && F <= WBG_DYN_SHC_RYOO && !field_ok(fs->S, 3, nFbar)) return WBG_ERR_ARG;
    if (F == WBG_DYN_SHC_QIAO &&
        !(field_ok(fs->SH, 3, nFbar) && field_ok(fs->SR, 9, nFbar) && field_ok(fs->SHR, 9, nFbar)))
      return WBG_ERR_ARG;
    if (F == WBG_DYN_SHC_RYOO && !(field_ok(fs->SA, 9, nFbar) && field_ok(fs->SHA, 9, nFbar))) return WBG_ERR_ARG;
    if (F == WBG_DYN_SHIFT && (!field_ok(fs->W, 9, nFbar) || (ext && !field_ok(fs->dA, 9, nFbar)) ||
                               !(fs->sc_eta > 0.0)))
      return WBG_ERR_ARG;
  }
  if (workspace_bytes < wbg_dynamic_workspace_bytes(F, nw, nk, kp->nEF)) return WBG_ERR_WORKSPACE;
  const int P = nw * nw;
  char* w = (char*)workspace;
  double* rec_dE = (double*)w; w += (size_t)nk * P * 8;
  void* rec_M = w; w += (size_t)nk * P * 16 * nc;
  void* rec_fE = w; w += (size_t)nk * P * 8 * kp->nEF;
  int* count = (int*)w;
  const size_t smp = (size_t)nw * 16 + (size_t)(2 * nw + 1) * 4;
  if (fp64)
    launch_pairs<double>(F, nk, smp, stream, E, Xbar, nFbar, *fs, nw, *kp, efermi, rec_dE, rec_fE, rec_M, count, P);
  else
    launch_pairs<float>(F, nk, smp, stream, E, Xbar, nFbar, *fs, nw, *kp, efermi, rec_dE, rec_fE, rec_M, count, P);
  // threads per block and levels per block: fewest passes over the records
  // (frequency blocks x level chunks), accumulators within 96 KB of shared memory
  const size_t smax = 96 * 1024;
  const size_t vsz = fp64 ? 16 : 8;  // one complex accumulator
  int tpb = 0, efc = 0;
  long long best = -1;
  for (int t = 128; t >= 32; t /= 2) {
    const int e = (int)((size_t)smax / ((size_t)t * nc * vsz));
    if (e < 1) continue;
    const int ec = e < kp->nEF ? e : kp->nEF;
    const long long passes = (long long)((kp->nOmega + t - 1) / t) * ((kp->nEF + ec - 1) / ec);
    if (best < 0 || passes < best) { best = passes; tpb = t; efc = ec; }
  }
  if (tpb == 0) return WBG_ERR_SIZE;
  const size_t sma = (size_t)tpb * efc * nc * vsz;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int wblocks = (kp->nOmega + tpb - 1) / tpb;
  const int eblocks = (kp->nEF + efc - 1) / efc;
  int nchunks = (4 * sms + wblocks * eblocks - 1) / (wblocks * eblocks);
  if (nchunks > nk) nchunks = nk;
  const int kchunk = (nk + nchunks - 1) / nchunks;
  nchunks = (nk + kchunk - 1) / kchunk;
  const dim3 grid(wblocks, nchunks, eblocks);
#define WBG_ACCUM(NC, R)                                                                                       \
  do {                                                                                                         \
    cudaFuncSetAttribute(kubo_accum<NC, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax);           \
    kubo_accum<NC, R><<<grid, tpb, sma, stream>>>(rec_dE, (const R*)rec_fE, (const typename C2<R>::t*)rec_M,   \
                                                 count, P, nk, kchunk, omega, *kp, F, efc, (wbg_u64*)out);     \
  } while (0)
  if (fp64) {
    if (nc == 1) WBG_ACCUM(1, double);
    else if (nc == 9) WBG_ACCUM(9, double);
    else WBG_ACCUM(27, double);
  } else if (nc == 1) {
    WBG_ACCUM(1, float);
  } else if (wbg_tuned(WBG_TUNE_KUBO_ENGINE, 0, 1) != 2) {  // tensor cores (the built-in choice)
    const int st = wbg_kubo_tc_run(rec_dE, rec_fE, rec_M, count, P, nk, omega, kp->nOmega, kp->nEF, nc, kp->eta,
                                   kp->gaussian, F, out, stream);
    if (st != WBG_OK) return st;
  } else {  // the register-tiled GEMM: one block per SM, frequency x column tiles x k chunks
    const int gw = (kp->nOmega + KG_TW - 1) / KG_TW, gc = (kp->nEF * nc + KG_TC - 1) / KG_TC;
    int gk = sms / (gw * gc);  // one wave of one block per SM
    if (gk < 1) gk = 1;
    if (gk > nk) gk = nk;
    const int kc = (nk + gk - 1) / gk;
    gk = (nk + kc - 1) / kc;
    const dim3 gg(gw, gk, gc);
    if (nc == 9) {
      cudaFuncSetAttribute(kubo_gemm<9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KG_SMEM);
      kubo_gemm<9><<<gg, KG_THR, KG_SMEM, stream>>>(rec_dE, (const float*)rec_fE, (const float2*)rec_M, count, P, nk,
                                                    kc, omega, *kp, F, (wbg_u64*)out);
    } else {
      cudaFuncSetAttribute(kubo_gemm<27>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KG_SMEM);
      kubo_gemm<27><<<gg, KG_THR, KG_SMEM, stream>>>(rec_dE, (const float*)rec_fE, (const float2*)rec_M, count, P, nk,
                                                     kc, omega, *kp, F, (wbg_u64*)out);
    }
  }
#undef WBG_ACCUM
  return wbg_cuda_status(cudaGetLastError());
}

size_t wbg_kubo_workspace_bytes(int nw, int nk, int nEF) {
  return wbg_dynamic_workspace_bytes(WBG_DYN_OPTCOND, nw, nk, nEF);
}

int wbg_kubo_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int nw, int nk, int external_terms,
                 const WbgKubo* kp, const double* efermi, const double* omega, void* workspace,
                 size_t workspace_bytes, void* out, int fp64, cudaStream_t stream) {
  if (!kp || kp->nEF > 64) return WBG_ERR_ARG;
  wbg_dynamic_spec fs = {};
  fs.formula = WBG_DYN_OPTCOND;
  fs.external_terms = external_terms ? 1 : 0;
  fs.V = iV;
  fs.A = iA;
  fs.W = fs.dA = fs.S = fs.SH = fs.SA = fs.SHA = fs.SR = fs.SHR = -1;
  return wbg_dynamic_run(E, Xbar, nFbar, &fs, nw, nk, kp, efermi, omega, workspace, workspace_bytes, out, fp64,
                         stream);
}
