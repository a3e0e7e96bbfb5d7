// R -> k transform of real-space matrices on one or more FFT blocks (stage 1 of the path).
//
// Replaces fourier/fft.py:133-192 (scatter + ifftn), fourier/rvectors.py:477-506
// (expdK phase, derivative i(R + t_n - t_m)) and data_K/data_K_R.py:28-51,91-97
// (rotAA and the R-space matrices behind Xbar).
//
// Two parts:
//  * r2k_weights (once per system and field set): the R-space derivative / curl weights of
//    rvectors.py:487-494 and data_K_R.py:48-51 applied to the base matrices, giving one
//    R-space array per k-space field, XF[f][R][mn] -- the reference does the same in R-space
//    before its FFT.
//  * the per-block transform X(k_j) = sum_R exp(2 pi i R.(j/N + dK)) XF_R as a pruned
//    separable DFT over the R-vectors actually present (sorted by (R0,R1,R2)):
//      stage A: contract R2 inside each (R0,R1) "pair"   -> Z[blk][f][pair][k2]
//      stage B: contract R1 inside each R0 "slice"       -> Y[blk][f][slice][k1][k2]
//      stage C: contract R0                              -> out[blk*nk + k][f]
//    Each thread keeps the (<= MAXL) inputs of its matrix elements in registers and loops
//    over the output index; the per-axis phase tables are broadcast from shared memory.
//    A thread owns one "column" (field f, element mn).  An optional column list restricts the
//    transform to a subset of elements -- the lower triangle of fields that are Hermitian by
//    construction, whose upper triangle the consumers mirror -- so the result is exactly
//    Hermitian and costs about half.
#include <type_traits>
#include "wbgpu_common.cuh"
#include "wbgpu_df64.cuh"
#include "wbgpu_r2k.cuh"

namespace {

constexpr int kThreads = 128;

// ---------------- R-space weights (once per system + field set) ----------------
// grid: ceil(nR*nw2/256) blocks; one thread per (R, m, n) computes the Cartesian weight
// R + t_n - t_m once (FP64) and writes every field.  XR [nBase][nR][nw2]; iR [nR][3] (sorted).
// XFlo (split precision, T = float): the rounding residual XF_R - float(XF_R), so that the
// k-independent R-space data carry 48 bits into the transform.
template <typename T>
__global__ void r2k_weights(const double2* __restrict__ XR, const int* __restrict__ iR, const int4* __restrict__ fdesc,
                            int nF, const double* __restrict__ wcc, R2KLattice lat, int nBase, int nR, int nw,
                            typename C2<T>::t* __restrict__ XF, typename C2<T>::t* __restrict__ XFlo) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nw2 = nw * nw;
  if (idx >= (long long)nR * nw2) return;
  const int r = (int)(idx / nw2), mn = (int)(idx % nw2);
  const int m = mn / nw, n = mn % nw;
  // R + t_n - t_m (Cartesian), rvectors.py:355-360
  double w[3];
  for (int a = 0; a < 3; ++a)
    w[a] = iR[r * 3 + 0] * lat.L[0 * 3 + a] + iR[r * 3 + 1] * lat.L[1 * 3 + a] + iR[r * 3 + 2] * lat.L[2 * 3 + a] +
           wcc[n * 3 + a] - wcc[m * 3 + a];
  for (int f = 0; f < nF; ++f) {
    const int4 fd = fdesc[f];
    const bool idx_ok = fd.z >= 0 && fd.z < 3 && fd.w >= 0 && fd.w < 3 && fd.y >= 0;
    const bool ok = idx_ok && ((fd.x <= R2K_DER2 && fd.y < nBase) || (fd.x >= R2K_ROT && fd.y + 2 < nBase)) &&
                    fd.x >= 0 && fd.x <= R2K_DROT;
    double2 v = make_double2(0.0, 0.0);
    if (!ok) {
      v = make_double2(0.0 / 0.0, 0.0 / 0.0);  // invalid descriptor: NaN, no out-of-range read
    } else if (fd.x == R2K_MOM0) {
      v = XR[((long long)fd.y * nR + r) * nw2 + mn];
    } else if (fd.x == R2K_DER1) {  // i w_a X
      v = cmuli(cscale(XR[((long long)fd.y * nR + r) * nw2 + mn], w[fd.z]));
    } else if (fd.x == R2K_DER2) {  // -w_a w_b X
      v = cscale(XR[((long long)fd.y * nR + r) * nw2 + mn], -w[fd.z] * w[fd.w]);
    } else {
      // rotAA_g = i w_alpha A_beta - i w_beta A_alpha, (alpha, beta) = ((1,2),(2,0),(0,1))[g]
      const int al = (fd.z + 1) % 3, be = (fd.z + 2) % 3;
      const double2 Ab = XR[((long long)(fd.y + be) * nR + r) * nw2 + mn];
      const double2 Aa = XR[((long long)(fd.y + al) * nR + r) * nw2 + mn];
      v = cmuli(csub(cscale(Ab, w[al]), cscale(Aa, w[be])));
      if (fd.x == R2K_DROT) v = cmuli(cscale(v, w[fd.w]));  // derivative of the curl
    }
    const typename C2<T>::t h = mkc<T>(real_from_double<T>(v.x), real_from_double<T>(v.y));
    XF[((long long)f * nR + r) * nw2 + mn] = h;
    if constexpr (std::is_same<T, float>::value)
      if (XFlo) XFlo[((long long)f * nR + r) * nw2 + mn] = mkc<T>((T)(v.x - (double)h.x), (T)(v.y - (double)h.y));
  }
}

// Column c of the launch -> (field, element).  cols == nullptr: all nF * nw2 columns.
WBG_D bool decode_col(const int* cols, int ncols, int nF, int nw2, int& f, int& mn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return false;
  const int fm = cols ? cols[c] : c;
  if (fm < 0 || fm >= nF * nw2) return false;  // list lives in device memory: validate here
  f = fm / nw2;
  mn = fm % nw2;
  return true;
}

// Phase tables in shared memory, transposed for the contraction: row r (an R index), Nj
// columns padded to JP = 4 ceil(Nj / 4).  FP32 entries are float4 (t.x, t.x, -t.y, t.y): the
// two register pairs of one 16-byte load feed the two packed FMAs of acc += t x
// (acc = (t.x, t.x) (x.x, x.y) + acc, then (-t.y, t.y) (x.y, x.x) + acc -- the same two
// roundings per component, in the same order, as four scalar FMAs).
template <typename T> struct PhaseEntry { typedef typename C2<T>::t type; };
template <> struct PhaseEntry<float> { typedef float4 type; };

template <typename T> WBG_D typename PhaseEntry<T>::type make_entry(typename C2<T>::t t) { return t; }
template <> WBG_D float4 make_entry<float>(float2 t) { return make_float4(t.x, t.x, -t.y, t.y); }

WBG_HD int pad4(int n) { return (n + 3) & ~3; }

template <typename T>
WBG_D void load_phases(const typename C2<T>::t* __restrict__ ph, int Nj, int nr,
                       typename PhaseEntry<T>::type* tabT) {
  typedef typename C2<T>::t V;
  const int JP = pad4(Nj);
  for (int idx = threadIdx.x; idx < nr * JP; idx += blockDim.x) {
    const int r = idx / JP, j = idx % JP;
    tabT[idx] = make_entry<T>(j < Nj ? ph[j * nr + r] : czero<V>());
  }
}

// acc += t x (xs = (x.y, x.x), used by the packed FP32 form); pdone ends an accumulation chain
template <typename T>
WBG_D void pmac(typename C2<T>::t& acc, const typename PhaseEntry<T>::type& t, typename C2<T>::t x,
                typename C2<T>::t xs) {
  cfma(acc, t, x);
}
template <typename T> WBG_D void pdone(typename C2<T>::t&) {}
// double-float: lazy chains (one renormalisation per output instead of one per term)
template <>
WBG_D void pmac<df64>(cdf& acc, const cdf& t, cdf x, cdf xs) {
  df_lazy_fma(acc.x, t.x, x.x);
  df_lazy_fma(acc.x, -t.y, x.y);
  df_lazy_fma(acc.y, t.x, x.y);
  df_lazy_fma(acc.y, t.y, x.x);
}
template <> WBG_D void pdone<df64>(cdf& a) {
  a.x = df_lazy_done(a.x);
  a.y = df_lazy_done(a.y);
}
template <>
WBG_D void pmac<float>(float2& acc, const float4& t, float2 x, float2 xs) {
  acc = __ffma2_rn(make_float2(t.x, t.y), x, acc);
  acc = __ffma2_rn(make_float2(t.z, t.w), xs, acc);
}

// One separable contraction: out[col][j] = sum_{i < len} tab[j][idx[i]] in[col][i]
// for every output index j < Nj, JB outputs per pass (independent accumulators, the sum over
// i in order): 4 for FP32, 1 for the 16-byte types, whose accumulators cost occupancy.
// `in` values of this thread stay in registers.
// Stored element: the transform's own type, or complex64 rounded from double-float (the mixed
// path's fields transformed in double-float, rounded once).
template <typename VO, typename V> WBG_D VO store_out(V a) { return a; }
template <> WBG_D float2 store_out<float2, cdf>(cdf a) { return make_float2(a.x.hi + a.x.lo, a.y.hi + a.y.lo); }

template <typename T, int MAXL, typename VO = typename C2<T>::t>
WBG_D void contract(const typename C2<T>::t* x, int len, const typename PhaseEntry<T>::type* tabT, const int* ridx,
                    int Nj, VO* out, long long out_stride) {
  typedef typename C2<T>::t V;
  typedef typename PhaseEntry<T>::type E;
  constexpr int JB = std::is_same<T, float>::value ? 4 : 1;
  const int JP = pad4(Nj);
  V xs[MAXL];
#pragma unroll
  for (int i = 0; i < MAXL; ++i) {
    xs[i].x = x[i].y;
    xs[i].y = x[i].x;
  }
  for (int j0 = 0; j0 < Nj; j0 += JB) {
    V a[JB];
#pragma unroll
    for (int q = 0; q < JB; ++q) a[q] = czero<V>();
#pragma unroll
    for (int i = 0; i < MAXL; ++i)
      if (i < len) {
        const E* t = tabT + ridx[i] * JP + j0;
#pragma unroll
        for (int q = 0; q < JB; ++q) pmac<T>(a[q], t[q], x[i], xs[i]);
      }
#pragma unroll
    for (int q = 0; q < JB; ++q) {
      pdone<T>(a[q]);
      if (j0 + q < Nj) out[(long long)(j0 + q) * out_stride] = store_out<VO>(a[q]);
    }
  }
}

// ---------------- stage A: contract R2 inside each (R0,R1) pair ----------------
// grid: (ceil(nF*nw2/kThreads), nP, nb); XF [nF][nR][nw2] -> Z [nb][nF][nP][N2][nw2]
template <typename T, int MAXL, bool SPLIT>
__global__ void __launch_bounds__(kThreads) r2k_stageA(const typename C2<T>::t* __restrict__ XF,
                                                       const typename C2<T>::t* __restrict__ XFlo,
                                                       const int* __restrict__ pairStart, const int* __restrict__ r2,
                                                       const typename C2<T>::t* __restrict__ ph2,
                                                       typename C2<T>::t* __restrict__ Z, R2KGeom g, int nF,
                                                       const int* __restrict__ cols, int ncols) {
  typedef typename C2<T>::t V;
  typedef typename PhaseEntry<T>::type E;
  extern __shared__ __align__(16) unsigned char smr[];
  E* tab = reinterpret_cast<E*>(smr);  // [nr2][pad4(N2)]
  const int p = blockIdx.y, blk = blockIdx.z;
  load_phases<T>(ph2 + (long long)blk * g.N2 * g.nr2, g.N2, g.nr2, tab);
  __syncthreads();
  int f, mn;
  if (!decode_col(cols, ncols, nF, g.nw2, f, mn)) return;
  const int r0 = pairStart[p], len = pairStart[p + 1] - r0;
  V x[MAXL], xl[SPLIT ? MAXL : 1];
  int ri[MAXL];
#pragma unroll
  for (int i = 0; i < MAXL; ++i) {
    if (i < len) {
      x[i] = XF[((long long)f * g.nR + r0 + i) * g.nw2 + mn];
      if (SPLIT) xl[i] = XFlo[((long long)f * g.nR + r0 + i) * g.nw2 + mn];
      ri[i] = r2[r0 + i] - g.rmin2;
    } else {
      x[i] = czero<V>();
      if (SPLIT) xl[i] = czero<V>();
      ri[i] = 0;
    }
  }
  V* out = Z + ((((long long)blk * nF + f) * g.nP + p) * g.N2) * g.nw2 + mn;
  if (SPLIT) {  // sum_R tab (XF + XFlo): the residual products accumulate separately
    V xs[MAXL], xls[MAXL];
#pragma unroll
    for (int i = 0; i < MAXL; ++i) {
      xs[i].x = x[i].y;
      xs[i].y = x[i].x;
      xls[i].x = xl[SPLIT ? i : 0].y;
      xls[i].y = xl[SPLIT ? i : 0].x;
    }
    const int JP = pad4(g.N2);
    for (int j0 = 0; j0 < g.N2; j0 += 2) {
      V a0 = czero<V>(), l0 = czero<V>(), a1 = czero<V>(), l1 = czero<V>();
#pragma unroll
      for (int i = 0; i < MAXL; ++i)
        if (i < len) {
          const E* t = tab + ri[i] * JP + j0;
          pmac<T>(a0, t[0], x[i], xs[i]);
          pmac<T>(l0, t[0], xl[SPLIT ? i : 0], xls[i]);
          pmac<T>(a1, t[1], x[i], xs[i]);
          pmac<T>(l1, t[1], xl[SPLIT ? i : 0], xls[i]);
        }
      out[(long long)j0 * g.nw2] = cadd(a0, l0);
      if (j0 + 1 < g.N2) out[(long long)(j0 + 1) * g.nw2] = cadd(a1, l1);
    }
  } else {
    contract<T, MAXL>(x, len, tab, ri, g.N2, out, g.nw2);
  }
}

// ---------------- stage B: contract R1 inside each R0 slice ----------------
// grid: (ceil(nF*nw2/kThreads), nU*N2, nb); Z -> Y [nb][nF][nU][N1][N2][nw2]
template <typename T, int MAXL>
__global__ void __launch_bounds__(kThreads) r2k_stageB(const typename C2<T>::t* __restrict__ Z,
                                                       const int* __restrict__ sliceStart,
                                                       const int* __restrict__ pairR1,
                                                       const typename C2<T>::t* __restrict__ ph1,
                                                       typename C2<T>::t* __restrict__ Y, R2KGeom g, int nF,
                                                       const int* __restrict__ cols, int ncols) {
  typedef typename C2<T>::t V;
  typedef typename PhaseEntry<T>::type E;
  extern __shared__ __align__(16) unsigned char smr[];
  E* tab = reinterpret_cast<E*>(smr);  // [nr1][pad4(N1)]
  const int u = blockIdx.y / g.N2, k2 = blockIdx.y % g.N2, blk = blockIdx.z;
  load_phases<T>(ph1 + (long long)blk * g.N1 * g.nr1, g.N1, g.nr1, tab);
  __syncthreads();
  int f, mn;
  if (!decode_col(cols, ncols, nF, g.nw2, f, mn)) return;
  const int p0 = sliceStart[u], len = sliceStart[u + 1] - p0;
  V x[MAXL];
  int ri[MAXL];
#pragma unroll
  for (int i = 0; i < MAXL; ++i) {
    if (i < len) {
      x[i] = Z[((((long long)blk * nF + f) * g.nP + p0 + i) * g.N2 + k2) * g.nw2 + mn];
      ri[i] = pairR1[p0 + i] - g.rmin1;
    } else {
      x[i] = czero<V>();
      ri[i] = 0;
    }
  }
  V* out = Y + (((((long long)blk * nF + f) * g.nU + u) * g.N1) * g.N2 + k2) * g.nw2 + mn;
  contract<T, MAXL>(x, len, tab, ri, g.N1, out, (long long)g.N2 * g.nw2);
}

// ---------------- stage C: contract R0 ----------------
// grid: (ceil(nF*nw2/kThreads), N1*N2, nb); Y -> out [nb*nk][nF][nw2]
template <typename T, int MAXL, typename VO>
__global__ void __launch_bounds__(kThreads) r2k_stageC(const typename C2<T>::t* __restrict__ Y,
                                                       const int* __restrict__ sliceR0,
                                                       const typename C2<T>::t* __restrict__ ph0,
                                                       VO* __restrict__ out, R2KGeom g, int nF,
                                                       const int* __restrict__ cols, int ncols) {
  typedef typename C2<T>::t V;
  typedef typename PhaseEntry<T>::type E;
  extern __shared__ __align__(16) unsigned char smr[];
  E* tab = reinterpret_cast<E*>(smr);  // [nr0][pad4(N0)]
  const int k1 = blockIdx.y / g.N2, k2 = blockIdx.y % g.N2, blk = blockIdx.z;
  load_phases<T>(ph0 + (long long)blk * g.N0 * g.nr0, g.N0, g.nr0, tab);
  __syncthreads();
  int f, mn;
  if (!decode_col(cols, ncols, nF, g.nw2, f, mn)) return;
  const int len = g.nU;
  V x[MAXL];
  int ri[MAXL];
#pragma unroll
  for (int i = 0; i < MAXL; ++i) {
    if (i < len) {
      x[i] = Y[(((((long long)blk * nF + f) * g.nU + i) * g.N1 + k1) * g.N2 + k2) * g.nw2 + mn];
      ri[i] = sliceR0[i] - g.rmin0;
    } else {
      x[i] = czero<V>();
      ri[i] = 0;
    }
  }
  const long long kstride = (long long)g.N1 * g.N2 * nF * g.nw2;  // k0 -> k0+1
  VO* o = out + (((long long)blk * g.nk + (long long)k1 * g.N2 + k2) * nF + f) * g.nw2 + mn;
  contract<T, MAXL, VO>(x, len, tab, ri, g.N0, o, kstride);
}

template <typename T, int MAXL, typename VO>
void launch_stages(const void* XF, const void* XFlo, int nF, const int* pairStart, const int* r2, const int* sliceStart,
                   const int* pairR1, const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, void* Z,
                   void* Y, void* out, const R2KGeom& g, int nb, const int* cols, int ncols, cudaStream_t stream) {
  typedef typename C2<T>::t V;
  typedef typename PhaseEntry<T>::type E;
  const unsigned colBlocks = (unsigned)((ncols + kThreads - 1) / kThreads);
  const size_t smA = (size_t)pad4(g.N2) * g.nr2 * sizeof(E), smB = (size_t)pad4(g.N1) * g.nr1 * sizeof(E),
               smC = (size_t)pad4(g.N0) * g.nr0 * sizeof(E);
  if (XFlo) {
    cudaFuncSetAttribute(r2k_stageA<T, MAXL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    r2k_stageA<T, MAXL, true><<<dim3(colBlocks, g.nP, nb), kThreads, smA, stream>>>(
        (const V*)XF, (const V*)XFlo, pairStart, r2, (const V*)ph2, (V*)Z, g, nF, cols, ncols);
  } else {
    cudaFuncSetAttribute(r2k_stageA<T, MAXL, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    r2k_stageA<T, MAXL, false><<<dim3(colBlocks, g.nP, nb), kThreads, smA, stream>>>(
        (const V*)XF, nullptr, pairStart, r2, (const V*)ph2, (V*)Z, g, nF, cols, ncols);
  }
  cudaFuncSetAttribute(r2k_stageB<T, MAXL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  r2k_stageB<T, MAXL><<<dim3(colBlocks, g.nU * g.N2, nb), kThreads, smB, stream>>>(
      (const V*)Z, sliceStart, pairR1, (const V*)ph1, (V*)Y, g, nF, cols, ncols);
  cudaFuncSetAttribute(r2k_stageC<T, MAXL, VO>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  r2k_stageC<T, MAXL, VO><<<dim3(colBlocks, g.N1 * g.N2, nb), kThreads, smC, stream>>>(
      (const V*)Y, sliceR0, (const V*)ph0, (VO*)out, g, nF, cols, ncols);
}

template <typename T, typename VO = typename C2<T>::t>
int launch_r2k(const void* XF, const void* XFlo, int nF, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
               const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, void* Z, void* Y, void* out,
               const R2KGeom& g, int nb, const int* cols, int ncols, cudaStream_t stream) {
  const int maxlen = max(max(g.maxPairLen, g.maxSliceLen), g.nU);
  if (maxlen <= 8)
    launch_stages<T, 8, VO>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, g, nb, cols,
                         ncols, stream);
  else if (maxlen <= 12)
    launch_stages<T, 12, VO>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, g, nb, cols,
                          ncols, stream);
  else if (maxlen <= 16)
    launch_stages<T, 16, VO>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, g, nb, cols,
                         ncols, stream);
  else if (maxlen <= 24)
    launch_stages<T, 24, VO>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, g, nb, cols,
                         ncols, stream);
  else if (maxlen <= WBG_R2K_MAXLEN)
    launch_stages<T, WBG_R2K_MAXLEN, VO>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, g,
                                     nb, cols, ncols, stream);
  else
    return WBG_ERR_SIZE;
  return wbg_cuda_status(cudaGetLastError());
}

}  // namespace

// prec: 0 FP32, 1 FP64, 2 double-float, 3 FP32 with R-space residuals, 4 double-float transform
// stored as complex64 (workspace and inputs as prec 2)
size_t wbg_r2k_workspace_bytes(const R2KGeom* g, int nF, int nb, int prec) {
  const size_t cs = (prec == 1 || prec == 2 || prec == 4) ? 16 : 8;
  const size_t z = (size_t)nb * nF * g->nP * g->N2 * g->nw2 * cs;
  const size_t y = (size_t)nb * nF * g->nU * g->N1 * g->N2 * g->nw2 * cs;
  return ((z + 255) / 256) * 256 + y;
}

int wbg_r2k_fields_run(const void* XR, int nBase, const int* iRsorted, int nR, int nw, const int4* fdesc, int nF,
                       const double* wcc, const R2KLattice* lat, int prec, void* XF, cudaStream_t stream) {
  if (!XR || !iRsorted || !fdesc || !wcc || !lat || !XF || nBase < 1 || nR < 1 || nw < 1 || nF < 1)
    return WBG_ERR_ARG;
  const long long n = (long long)nR * nw * nw;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (prec < 0 || prec > 3) return WBG_ERR_ARG;
  if (prec == 1)
    r2k_weights<double><<<grid, 256, 0, stream>>>((const double2*)XR, iRsorted, fdesc, nF, wcc, *lat, nBase, nR, nw,
                                                  (double2*)XF, nullptr);
  else if (prec == 2)
    r2k_weights<df64><<<grid, 256, 0, stream>>>((const double2*)XR, iRsorted, fdesc, nF, wcc, *lat, nBase, nR, nw,
                                                (cdf*)XF, nullptr);
  else  // prec 3: residuals right after the rounded values
    r2k_weights<float><<<grid, 256, 0, stream>>>((const double2*)XR, iRsorted, fdesc, nF, wcc, *lat, nBase, nR, nw,
                                                 (float2*)XF, prec == 3 ? (float2*)XF + n * nF : nullptr);
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_r2k_run(const void* XF, int nF, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
                const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, void* workspace,
                size_t workspace_bytes, void* out, const R2KGeom* g, int nb, int prec, const int* cols, int ncols,
                cudaStream_t stream) {
  if (!g || nF <= 0 || nb <= 0 || prec < 0 || prec > 4) return WBG_ERR_ARG;
  if (!cols) ncols = nF * g->nw2;
  if (ncols < 1 || ncols > nF * g->nw2) return WBG_ERR_ARG;
  if (g->nw2 != g->nw * g->nw || g->nk != g->N0 * g->N1 * g->N2) return WBG_ERR_ARG;
  if (g->nU < 1 || g->nP < 1 || g->maxPairLen < 1 || g->maxSliceLen < 1) return WBG_ERR_ARG;
  if (workspace_bytes < wbg_r2k_workspace_bytes(g, nF, nb, prec)) return WBG_ERR_WORKSPACE;
  const size_t cs = (prec == 1 || prec == 2 || prec == 4) ? 16 : 8;
  const size_t z = (size_t)nb * nF * g->nP * g->N2 * g->nw2 * cs;
  char* Z = (char*)workspace;
  char* Y = Z + ((z + 255) / 256) * 256;
  if (prec == 1)
    return launch_r2k<double>(XF, nullptr, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, *g, nb,
                              cols, ncols, stream);
  if (prec == 2)
    return launch_r2k<df64>(XF, nullptr, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, *g, nb,
                            cols, ncols, stream);
  if (prec == 4)
    return launch_r2k<df64, float2>(XF, nullptr, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y,
                                    out, *g, nb, cols, ncols, stream);
  const void* XFlo = prec == 3 ? (const void*)((const float2*)XF + (size_t)nF * g->nR * g->nw2) : nullptr;
  return launch_r2k<float>(XF, XFlo, nF, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, Z, Y, out, *g, nb,
                           cols, ncols, stream);
}
