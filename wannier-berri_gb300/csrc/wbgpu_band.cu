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
#include "wbgpu_band.cuh"

namespace {

// ---------------------------------------------------------------------------------------
// rotation: Xbar[k][f] = U^dagger X[k][fsel[f]] U  (optionally Hermitian-symmetrised)
// grid: nk blocks of 256 threads; shared: U, X, T (nw*nw each, precision T)
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void rotate_kernel(const typename C2<T>::t* __restrict__ U, long long strideU, const typename C2<T>::t* __restrict__ X,
                              int nFin, const int* __restrict__ fsel, const int* __restrict__ herm, int nFrot,
                              typename C2<T>::t* __restrict__ Xbar, int nw) {
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
    const T nan = T(0) / T(0);
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) Xs[i] = fok ? src[i] : mkc<T>(nan, nan);
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
    V* dst = Xbar + (k * nFrot + f) * (long long)nw2;
    const bool h = herm[f] != 0;
    for (int i = threadIdx.x; i < nw2; i += blockDim.x) {
      V y = Xs[i];
      if (h) {
        const int m = i / nw, n = i % nw;
        const V yt = Xs[n * nw + m];
        y = mkc<T>((T)0.5 * (y.x + yt.x), (T)0.5 * (y.y - yt.y));
      }
      dst[i] = y;
    }
    __syncthreads();
  }
}

// Register-tiled rotation for nw % 4 == 0: each thread owns a 4x4 tile of the nw x nw
// output; KB k-points per CTA.  X rows are padded (stride nw+1) so the column reads of
// different tile rows fall in different banks.  Same math as rotate_kernel.
template <typename T>
__global__ void rotate_tiled(const typename C2<T>::t* __restrict__ U, long long strideU,
                             const typename C2<T>::t* __restrict__ X, int nFin, const int* __restrict__ fsel,
                             const int* __restrict__ herm, int nFrot, typename C2<T>::t* __restrict__ Xbar, int nw,
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
    const T nan = T(0) / T(0);
    for (int i = tid; i < nw2; i += tpk) Xs[(i / nw) * ldx + (i % nw)] = fok ? src[i] : mkc<T>(nan, nan);
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
    V* dst = Xbar + (k * nFrot + f) * (long long)nw2;
    const bool h = herm[f] != 0;
    if (valid) {
      for (int i = tid; i < nw2; i += tpk) {
        const int m = i / nw, n = i % nw;
        V y = Xs[m * ldx + n];
        if (h) {
          const V yt = Xs[n * ldx + m];
          y = mkc<T>((T)0.5 * (y.x + yt.x), (T)0.5 * (y.y - yt.y));
        }
        dst[i] = y;
      }
    }
    __syncthreads();
  }
}

WBG_D int group_sum_i(int v, int L) {
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

// ---------------------------------------------------------------------------------------
// Fused Omega traces + Fermi-level histogram.
// grid: persistent blocks of G*L threads; each group of L lanes takes one k-point at a time.
// Xbar layout: [k][nFbar][nw][nw]; V at iV..iV+2, A at iA..iA+2, O(rotAA) at iO..iO+2.
// hist: [nEF][3] doubles, accumulated with atomics (FP64).
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void berry_omega_kernel(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar,
                                   int iV, int iA, int iO, int nw, int nk, int L, int G, WbgScan sp, int internal_terms,
                                   int external_terms, double* __restrict__ hist) {
  typedef typename C2<T>::t V;
  extern __shared__ double smb[];
  double* sh = smb;                                   // [nEF][3]
  double* Es = sh + 3 * sp.nEF;                       // [G][nw]
  double* tv = Es + G * nw;                           // [G][nw][3]
  int* start = reinterpret_cast<int*>(tv + 3 * G * nw);  // [G][nw]
  for (int i = threadIdx.x; i < 3 * sp.nEF; i += blockDim.x) sh[i] = 0.0;
  __syncthreads();
  const int grp = threadIdx.x / L, lane = threadIdx.x % L;
  double* myE = Es + grp * nw;
  double* myT = tv + 3 * grp * nw;
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
    const int bandmax = min(below, f0);
    const V* Xk = Xbar + kk * nFbar * nw2;
    for (int n = lane; n < nw; n += L) {
      int gs = n, ge = n + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      bool ingroup;
      if (n < bandmax) { gs = 0; ge = bandmax; ingroup = true; }
      else ingroup = (myE[ge - 1] >= sp.EFmin && myE[gs] <= sp.EFmax);
      double t[3] = {0.0, 0.0, 0.0};
      if (ingroup) {
        const double En = myE[n];
        double sr[3] = {0.0, 0.0, 0.0}, si[3] = {0.0, 0.0, 0.0};
        for (int l = 0; l < nw; ++l) {
          if (l >= gs && l < ge) continue;
          const double dE = En - myE[l];
          const T dinv = fabs(dE) < 1e-7 ? T(0) : recip_gap<T>(dE);
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
            // S += -i D^a_nl D^b_ln - D^a_nl A^b_ln + D^b_nl A^a_ln
            sr[g] += (double)(-acc.x) + (double)accx.x;
            si[g] += (double)(-acc.y) + (double)accx.y;
          }
        }
        if (external_terms) {
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            const int al = (g + 1) % 3, be = (g + 2) % 3;
            sr[g] += 0.5 * (double)Xk[(iO + g) * nw2 + n * nw + n].x;
            V acc = czero<V>();
            for (int np = gs; np < ge; ++np) cfma(acc, Xk[(iA + al) * nw2 + n * nw + np], Xk[(iA + be) * nw2 + np * nw + n]);
            // -i * acc
            sr[g] += (double)acc.y;
            si[g] -= (double)acc.x;
          }
        }
        for (int g = 0; g < 3; ++g) t[g] = 2.0 * sr[g];
      }
      for (int g = 0; g < 3; ++g) myT[n * 3 + g] = t[g];
    }
    __syncwarp();
    if (valid) {
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
          for (int g = 0; g < 3; ++g) atomicAdd(&sh[bin * 3 + g], v[g]);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * sp.nEF; i += blockDim.x)
    if (sh[i] != 0.0) atomicAdd(&hist[i], sh[i]);
}

// cumulative sum over Fermi levels and normalisation: out[ie][c] = scale * sum_{j<=ie} hist[j][c]
__global__ void scan_finalize_kernel(const double* __restrict__ hist, int nEF, int ncomp, double scale,
                                     double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncomp) return;
  double s = 0.0;
  for (int ie = 0; ie < nEF; ++ie) {
    s += hist[(long long)ie * ncomp + c];
    out[(long long)ie * ncomp + c] = s * scale;
  }
}

int lanes_for(int n) {
  int L = 1;
  while (L < n && L < 32) L <<= 1;
  return L < 4 ? 4 : L;
}

template <typename T>
int launch_rotate(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                  int nFrot, void* Xbar, int nw, int nk, cudaStream_t stream) {
  typedef typename C2<T>::t V;
  if (nw % 4 == 0 && nw >= 8) {
    const int tpk = (nw / 4) * (nw / 4);
    const size_t per_k = ((size_t)nw * nw * 2 + (size_t)nw * (nw + 1)) * sizeof(V);
    int KB = 1;
    while (KB * 2 * tpk <= 256 && (KB * 2) * per_k <= 64 * 1024) KB *= 2;
    if (KB * per_k <= 200 * 1024) {
      cudaFuncSetAttribute(rotate_tiled<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      rotate_tiled<T><<<(nk + KB - 1) / KB, KB * tpk, KB * per_k, stream>>>((const V*)U, strideU, (const V*)X, nFin,
                                                                           fsel, herm, nFrot, (V*)Xbar, nw, nk, KB);
      return wbg_cuda_status(cudaGetLastError());
    }
  }
  const size_t sm = 3 * (size_t)nw * nw * sizeof(V);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  cudaFuncSetAttribute(rotate_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  rotate_kernel<T><<<nk, 256, sm, stream>>>((const V*)U, strideU, (const V*)X, nFin, fsel, herm, nFrot, (V*)Xbar, nw);
  return wbg_cuda_status(cudaGetLastError());
}

}  // namespace

int wbg_rotate_run(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                   int nFrot, void* Xbar, int nw, int nk, int fp64, cudaStream_t stream) {
  if (nw < 1 || nk < 1 || nFrot < 1 || !U || !X || !Xbar || !fsel || !herm) return WBG_ERR_ARG;
  if (fp64) return launch_rotate<double>(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream);
  return launch_rotate<float>(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, stream);
}

int wbg_berry_omega_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                        const WbgScan* sp, int internal_terms, int external_terms, double* hist, int fp64,
                        cudaStream_t stream) {
  if (nw < 1 || nk < 1 || !sp || sp->nEF < 1 || !hist || !E || !Xbar) return WBG_ERR_ARG;
  if (iV < 0 || iV + 3 > nFbar) return WBG_ERR_ARG;
  if (external_terms && (iA < 0 || iA + 3 > nFbar || iO < 0 || iO + 3 > nFbar)) return WBG_ERR_ARG;
  if (!(sp->dEF > 0.0)) return WBG_ERR_ARG;
  const int L = lanes_for(nw);
  const int G = 128 / L;
  const size_t sm = 3 * (size_t)sp->nEF * 8 + (size_t)G * nw * (8 + 24 + 4);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nk + G - 1) / G;
  const long long cap = (long long)sms * 8;
  if (nblk > cap) nblk = cap;
  if (fp64) {
    cudaFuncSetAttribute(berry_omega_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_omega_kernel<double><<<(int)nblk, G * L, sm, stream>>>(E, (const double2*)Xbar, nFbar, iV, iA, iO, nw, nk, L,
                                                                 G, *sp, internal_terms, external_terms, hist);
  } else {
    cudaFuncSetAttribute(berry_omega_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    berry_omega_kernel<float><<<(int)nblk, G * L, sm, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, iO, nw, nk, L,
                                                                G, *sp, internal_terms, external_terms, hist);
  }
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_scan_finalize_run(const double* hist, int nEF, int ncomp, double scale, double* out, cudaStream_t stream) {
  if (nEF < 1 || ncomp < 1 || !hist || !out) return WBG_ERR_ARG;
  scan_finalize_kernel<<<(ncomp + 31) / 32, 32, 0, stream>>>(hist, nEF, ncomp, scale, out);
  return wbg_cuda_status(cudaGetLastError());
}
