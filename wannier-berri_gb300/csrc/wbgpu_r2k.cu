// R -> k transform of real-space matrices on one or more FFT blocks (stage 1 of the path).
//
// Replaces fourier/fft.py:133-192 (scatter + ifftn), fourier/rvectors.py:477-506
// (expdK phase, derivative i(R + t_n - t_m)) and data_K/data_K_R.py:28-51,91-97
// (rotAA, Xbar before rotation).
//
// X(k_j) = sum_R exp(2 pi i R.(j/N + dK)) w(R) X_R is evaluated as a pruned
// separable DFT over the R-vectors actually present (sorted by (R0,R1,R2)):
//   stage A: contract R2 for every (R0,R1) "pair"       -> Z[pair][k2]
//   stage B: contract R1 for every R0 "slice"           -> Y[slice][k1][k2]
//   stage C: contract R0, then build Cartesian fields   -> fields[k][f]
// Reduced-coordinate polynomial weights R_j, R_j R_l ride along each stage so that
// first and second k-derivatives come out as moments; stage C turns the moments into
// Cartesian derivatives with the Wannier-centre term (t_n - t_m) exactly as
// rvectors.py:355-369,487-494 define them.  The same code runs in FP64 and FP32.
#include "wbgpu_common.cuh"
#include "wbgpu_r2k.cuh"

namespace {

// moment q (0..9) -> (stage-B variant, power of R0); see header for the variant order
__constant__ int kMomB[3][10] = {{0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
                                 {0, 0, 1, 2, 0, 0, 0, 0, 0, 0},
                                 {0, 0, 1, 3, 0, 1, 3, 2, 4, 5}};
__constant__ int kMomE[3][10] = {{0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
                                 {0, 1, 0, 0, 0, 0, 0, 0, 0, 0},
                                 {0, 1, 0, 0, 2, 1, 1, 0, 0, 0}};
// stage-B variant v -> (stage-A variant, power of R1)
__constant__ int kVarA[3][6] = {{0, 0, 0, 0, 0, 0}, {0, 0, 1, 0, 0, 0}, {0, 0, 0, 1, 1, 2}};
__constant__ int kVarT[3][6] = {{0, 0, 0, 0, 0, 0}, {0, 1, 0, 0, 0, 0}, {0, 1, 2, 0, 1, 0}};

template <typename T>
WBG_D T ipow(int r, int e) {
  return e == 0 ? T(1) : (e == 1 ? T(r) : T(r) * T(r));
}

// ---------------- stage A: contract R2 inside each (R0,R1) pair ----------------
// grid: (nP, nb*nBase, ceil(nw2/TILE)); block: TILE threads (one per matrix element)
template <typename T>
__global__ void r2k_stageA(const typename C2<T>::t* __restrict__ X, const int* __restrict__ pairStart,
                           const int* __restrict__ r2, const typename C2<T>::t* __restrict__ ph2,
                           typename C2<T>::t* __restrict__ Z, R2KGeom g, int order) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smem_raw[];
  V* Xs = reinterpret_cast<V*>(smem_raw);
  const int p = blockIdx.x;
  const int blk = blockIdx.y / g.nBase, b = blockIdx.y % g.nBase;
  const int mn = blockIdx.z * blockDim.x + threadIdx.x;
  const int nA = order + 1;
  const int r0 = pairStart[p], len = pairStart[p + 1] - r0;
  if (mn < g.nw2) {
    for (int i = 0; i < len; ++i) Xs[i * blockDim.x + threadIdx.x] = X[((size_t)b * g.nR + r0 + i) * g.nw2 + mn];
  }
  __syncthreads();
  if (mn >= g.nw2) return;
  const V* ph = ph2 + (size_t)blk * g.N2 * g.nr2;
  for (int k2 = 0; k2 < g.N2; ++k2) {
    V acc[3] = {czero<V>(), czero<V>(), czero<V>()};
    for (int i = 0; i < len; ++i) {
      const int R2 = r2[r0 + i];
      V t = cmul(ph[k2 * g.nr2 + (R2 - g.rmin2)], Xs[i * blockDim.x + threadIdx.x]);
      acc[0] = cadd(acc[0], t);
      if (nA > 1) { cfma(acc[1], t, mkc<T>(T(R2), T(0))); }
      if (nA > 2) { cfma(acc[2], t, mkc<T>(T(R2) * T(R2), T(0))); }
    }
    for (int s = 0; s < nA; ++s)
      Z[((((size_t)blk * g.nBase + b) * nA + s) * g.nP + p) * ((size_t)g.N2 * g.nw2) + (size_t)k2 * g.nw2 + mn] = acc[s];
  }
}

// ---------------- stage B: contract R1 inside each R0 slice ----------------
// grid: (nU*N2, nb*nBase, tiles); block: TILE threads
template <typename T>
__global__ void r2k_stageB(const typename C2<T>::t* __restrict__ Z, const int* __restrict__ sliceStart,
                           const int* __restrict__ pairR1, const typename C2<T>::t* __restrict__ ph1,
                           typename C2<T>::t* __restrict__ Y, R2KGeom g, int order) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smem_raw[];
  V* Zs = reinterpret_cast<V*>(smem_raw);
  const int u = blockIdx.x / g.N2, k2 = blockIdx.x % g.N2;
  const int blk = blockIdx.y / g.nBase, b = blockIdx.y % g.nBase;
  const int mn = blockIdx.z * blockDim.x + threadIdx.x;
  const int nA = order + 1, nB = order == 0 ? 1 : (order == 1 ? 3 : 6);
  const int p0 = sliceStart[u], len = sliceStart[u + 1] - p0;
  const int TILE = blockDim.x;
  if (mn < g.nw2) {
    for (int s = 0; s < nA; ++s)
      for (int i = 0; i < len; ++i)
        Zs[(s * len + i) * TILE + threadIdx.x] =
            Z[((((size_t)blk * g.nBase + b) * nA + s) * g.nP + p0 + i) * ((size_t)g.N2 * g.nw2) + (size_t)k2 * g.nw2 + mn];
  }
  __syncthreads();
  if (mn >= g.nw2) return;
  const V* ph = ph1 + (size_t)blk * g.N1 * g.nr1;
  for (int k1 = 0; k1 < g.N1; ++k1) {
    V acc[6];
#pragma unroll
    for (int v = 0; v < 6; ++v) acc[v] = czero<V>();
    for (int i = 0; i < len; ++i) {
      const int R1 = pairR1[p0 + i];
      const V e = ph[k1 * g.nr1 + (R1 - g.rmin1)];
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        if (v < nB) {
          const int sa = kVarA[order][v], t = kVarT[order][v];
          V term = cmul(e, Zs[(sa * len + i) * TILE + threadIdx.x]);
          acc[v] = cadd(acc[v], cscale(term, ipow<T>(R1, t)));
        }
      }
    }
    const size_t plane = (size_t)g.N1 * g.N2 * g.nw2;
    for (int v = 0; v < nB; ++v)
      Y[((((size_t)blk * g.nBase + b) * nB + v) * g.nU + u) * plane + ((size_t)k1 * g.N2 + k2) * g.nw2 + mn] = acc[v];
  }
}

// Cartesian first / second moments from reduced ones (R_cart,a = sum_j iR_j L[j][a]).
template <typename T, typename V>
WBG_D V cart1(const V* M, const T* L, int a) {  // M[1..3] reduced first moments
  V r = czero<V>();
  for (int j = 0; j < 3; ++j) r = cadd(r, cscale(M[1 + j], L[j * 3 + a]));
  return r;
}
template <typename T, typename V>
WBG_D V cart2(const V* M, const T* L, int a, int b) {  // M[4..9] = 00,01,02,11,12,22
  const int idx[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
  V r = czero<V>();
  for (int j = 0; j < 3; ++j)
    for (int l = 0; l < 3; ++l) r = cadd(r, cscale(M[idx[j][l]], L[j * 3 + a] * L[l * 3 + b]));
  return r;
}
// d/dk_a X = i (C_a + d_a M0)
template <typename T, typename V>
WBG_D V der1(const V* M, const T* L, const T* d, int a) {
  return cmuli(cadd(cart1<T, V>(M, L, a), cscale(M[0], d[a])));
}
// d/dk_a d/dk_b X = -(C_ab + d_a C_b + d_b C_a + d_a d_b M0)
template <typename T, typename V>
WBG_D V der2(const V* M, const T* L, const T* d, int a, int b) {
  V r = cart2<T, V>(M, L, a, b);
  r = cadd(r, cscale(cart1<T, V>(M, L, b), d[a]));
  r = cadd(r, cscale(cart1<T, V>(M, L, a), d[b]));
  r = cadd(r, cscale(M[0], d[a] * d[b]));
  return cscale(r, T(-1));
}

// ---------------- stage C: contract R0 and emit Cartesian fields ----------------
// grid: (N1*N2, nb, tiles); block: TILE threads
template <typename T>
__global__ void r2k_stageC(const typename C2<T>::t* __restrict__ Y, const int* __restrict__ sliceR0,
                           const typename C2<T>::t* __restrict__ ph0, const int4* __restrict__ fdesc,
                           const T* __restrict__ wcc, typename C2<T>::t* __restrict__ out, R2KGeom g, int order,
                           int nF, R2KLattice lat) {
  typedef typename C2<T>::t V;
  extern __shared__ unsigned char smem_raw[];
  const int TILE = blockDim.x;
  const int nB = order == 0 ? 1 : (order == 1 ? 3 : 6);
  const int nM = order == 0 ? 1 : (order == 1 ? 4 : 10);
  V* Ys = reinterpret_cast<V*>(smem_raw);                          // [nBase*nB][nU][TILE]
  V* Ms = Ys + (size_t)g.nBase * nB * g.nU * TILE;                  // [nBase][nM][TILE]
  const int k1 = blockIdx.x / g.N2, k2 = blockIdx.x % g.N2;
  const int blk = blockIdx.y;
  const int mn = blockIdx.z * TILE + threadIdx.x;
  const bool active = mn < g.nw2;
  const size_t plane = (size_t)g.N1 * g.N2 * g.nw2;
  if (active) {
    for (int bv = 0; bv < g.nBase * nB; ++bv)
      for (int u = 0; u < g.nU; ++u)
        Ys[((size_t)bv * g.nU + u) * TILE + threadIdx.x] =
            Y[(((size_t)blk * g.nBase * nB + bv) * g.nU + u) * plane + ((size_t)k1 * g.N2 + k2) * g.nw2 + mn];
  }
  __syncthreads();
  if (!active) return;
  T L[9];
  for (int i = 0; i < 9; ++i) L[i] = (T)lat.L[i];
  const int m = mn / g.nw, n = mn % g.nw;
  T d[3];
  for (int a = 0; a < 3; ++a) d[a] = wcc[n * 3 + a] - wcc[m * 3 + a];
  const V* ph = ph0 + (size_t)blk * g.N0 * g.nr0;
  V* myM = Ms + threadIdx.x;
  for (int k0 = 0; k0 < g.N0; ++k0) {
    const size_t k = ((size_t)k0 * g.N1 + k1) * g.N2 + k2;
    for (int b = 0; b < g.nBase; ++b) {
      V acc[10];
#pragma unroll
      for (int q = 0; q < 10; ++q) acc[q] = czero<V>();
      for (int u = 0; u < g.nU; ++u) {
        const int R0 = sliceR0[u];
        const V e = ph[k0 * g.nr0 + (R0 - g.rmin0)];
        const T r = T(R0);
#pragma unroll
        for (int q = 0; q < 10; ++q) {
          if (q < nM) {
            V t = cmul(e, Ys[((size_t)(b * nB + kMomB[order][q]) * g.nU + u) * TILE + threadIdx.x]);
            const int ee = kMomE[order][q];
            if (ee >= 1) t = cscale(t, r);
            if (ee >= 2) t = cscale(t, r);
            acc[q] = cadd(acc[q], t);
          }
        }
      }
      for (int q = 0; q < nM; ++q) myM[((size_t)b * nM + q) * TILE] = acc[q];
    }
    // epilogue: build the requested fields for element (m, n)
    V Mb[10], Mc[10];
    for (int f = 0; f < nF; ++f) {
      const int4 fd = fdesc[f];
      V val = czero<V>();
      // descriptors live in device memory: validate here, emit NaN for an invalid one
      const bool idx_ok = fd.z >= 0 && fd.z < 3 && fd.w >= 0 && fd.w < 3 && fd.y >= 0;
      const bool ok = idx_ok && ((fd.x == R2K_MOM0 && fd.y < g.nBase) ||
                                 (fd.x == R2K_DER1 && order >= 1 && fd.y < g.nBase) ||
                                 (fd.x == R2K_DER2 && order >= 2 && fd.y < g.nBase) ||
                                 (fd.x == R2K_ROT && order >= 1 && fd.y + 2 < g.nBase) ||
                                 (fd.x == R2K_DROT && order >= 2 && fd.y + 2 < g.nBase));
      if (!ok) {
        const T nan = T(0) / T(0);
        val = mkc<T>(nan, nan);
      } else if (fd.x == R2K_MOM0) {
        val = myM[((size_t)fd.y * nM + 0) * TILE];
      } else if (fd.x == R2K_DER1) {
        for (int q = 0; q < 4; ++q) Mb[q] = myM[((size_t)fd.y * nM + q) * TILE];
        val = der1<T, V>(Mb, L, d, fd.z);
      } else if (fd.x == R2K_DER2) {
        for (int q = 0; q < 10; ++q) Mb[q] = myM[((size_t)fd.y * nM + q) * TILE];
        val = der2<T, V>(Mb, L, d, fd.z, fd.w);
      } else if (fd.x == R2K_ROT || fd.x == R2K_DROT) {
        // rotAA_g = d_alpha A_beta - d_beta A_alpha with (alpha, beta) = ((1,2),(2,0),(0,1))[g]
        const int al = (fd.z + 1) % 3, be = (fd.z + 2) % 3;
        const int nq = fd.x == R2K_ROT ? 4 : 10;
        for (int q = 0; q < nq; ++q) {
          Mb[q] = myM[((size_t)(fd.y + be) * nM + q) * TILE];
          Mc[q] = myM[((size_t)(fd.y + al) * nM + q) * TILE];
        }
        if (fd.x == R2K_ROT)
          val = csub(der1<T, V>(Mb, L, d, al), der1<T, V>(Mc, L, d, be));
        else
          val = csub(der2<T, V>(Mb, L, d, fd.w, al), der2<T, V>(Mc, L, d, fd.w, be));
      }
      out[((size_t)blk * g.nk + k) * ((size_t)nF * g.nw2) + (size_t)f * g.nw2 + mn] = val;
    }
  }
}

template <typename T>
int launch_r2k(const void* X, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
               const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, const int4* fdesc,
               const void* wcc, void* Z, void* Y, void* out, const R2KGeom& g, int order, int nF,
               const R2KLattice& lat, int nb, cudaStream_t stream) {
  typedef typename C2<T>::t V;
  const int nA = order + 1, nB = order == 0 ? 1 : (order == 1 ? 3 : 6);
  const int nM = order == 0 ? 1 : (order == 1 ? 4 : 10);
  // tile sizes: largest power of two <= 64 whose shared-memory footprint fits
  int tileC = 64;
  auto smemC = [&](int t) { return (size_t)t * sizeof(V) * ((size_t)g.nBase * nB * g.nU + (size_t)g.nBase * nM); };
  while (tileC > 8 && smemC(tileC) > 200 * 1024) tileC /= 2;
  if (smemC(tileC) > 220 * 1024) return WBG_ERR_SIZE;
  const int tileA = 64, tileB = 64;
  const size_t smemA = (size_t)tileA * g.maxPairLen * sizeof(V);
  const size_t smemB = (size_t)tileB * nA * g.maxSliceLen * sizeof(V);
  if (smemA > 220 * 1024 || smemB > 220 * 1024) return WBG_ERR_SIZE;
  cudaFuncSetAttribute(r2k_stageA<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  cudaFuncSetAttribute(r2k_stageB<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  cudaFuncSetAttribute(r2k_stageC<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  dim3 gA(g.nP, nb * g.nBase, (g.nw2 + tileA - 1) / tileA);
  r2k_stageA<T><<<gA, tileA, smemA, stream>>>((const V*)X, pairStart, r2, (const V*)ph2, (V*)Z, g, order);
  dim3 gB(g.nU * g.N2, nb * g.nBase, (g.nw2 + tileB - 1) / tileB);
  r2k_stageB<T><<<gB, tileB, smemB, stream>>>((const V*)Z, sliceStart, pairR1, (const V*)ph1, (V*)Y, g, order);
  dim3 gC(g.N1 * g.N2, nb, (g.nw2 + tileC - 1) / tileC);
  r2k_stageC<T><<<gC, tileC, smemC(tileC), stream>>>((const V*)Y, sliceR0, (const V*)ph0, fdesc, (const T*)wcc,
                                                     (V*)out, g, order, nF, lat);
  return wbg_cuda_status(cudaGetLastError());
}

}  // namespace

size_t wbg_r2k_workspace_bytes(const R2KGeom* g, int order, int nb, int fp64) {
  const size_t cs = fp64 ? sizeof(double2) : sizeof(float2);
  const int nA = order + 1, nB = order == 0 ? 1 : (order == 1 ? 3 : 6);
  const size_t z = (size_t)nb * g->nBase * nA * g->nP * g->N2 * g->nw2 * cs;
  const size_t y = (size_t)nb * g->nBase * nB * g->nU * g->N1 * g->N2 * g->nw2 * cs;
  return ((z + 255) / 256) * 256 + y;
}

int wbg_r2k_run(const void* X, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
                const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, const int4* fdesc,
                const void* wcc, void* workspace, size_t workspace_bytes, void* out, const R2KGeom* g, int order,
                int nF, const R2KLattice* lat, int nb, int fp64, cudaStream_t stream) {
  if (!g || !lat || order < 0 || order > 2 || nF <= 0 || nb <= 0) return WBG_ERR_ARG;
  if (g->nw2 != g->nw * g->nw || g->nk != g->N0 * g->N1 * g->N2) return WBG_ERR_ARG;
  const size_t need = wbg_r2k_workspace_bytes(g, order, nb, fp64);
  if (workspace_bytes < need) return WBG_ERR_WORKSPACE;
  const size_t cs = fp64 ? sizeof(double2) : sizeof(float2);
  const int nA = order + 1;
  const size_t z = (size_t)nb * g->nBase * nA * g->nP * g->N2 * g->nw2 * cs;
  char* Z = (char*)workspace;
  char* Y = Z + ((z + 255) / 256) * 256;
  if (fp64)
    return launch_r2k<double>(X, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, fdesc, wcc, Z, Y, out,
                              *g, order, nF, *lat, nb, stream);
  return launch_r2k<float>(X, pairStart, r2, sliceStart, pairR1, sliceR0, ph0, ph1, ph2, fdesc, wcc, Z, Y, out, *g,
                           order, nF, *lat, nb, stream);
}
