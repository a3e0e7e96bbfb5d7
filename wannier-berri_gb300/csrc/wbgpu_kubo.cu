// Kubo optical conductivity (stage 4, dynamic calculators).
//
// Replaces calculators/dynamic.py:71-114 (DynamicCalculator.__call__), 170-181
// (Formula_OptCond) and 184-196 (OpticalConductivity.factor_omega):
//   restot[E_F][w][a][b] += sum_{group pairs} f_w(E1,E2) f_E(E1,E2) M^{ab}_{12}
//   M^{ab}_{12} = sum_{n in G1, m in G2} i A^a_nm A^b_mn,   A = i D + Abar (data_K.py:328-334)
//   f_E = FD(E2) - FD(E1),   f_w = (E2 - E1) / (E2 - E1 - w - i eta)  (Lorentzian; for the
//   Gaussian smearing the imaginary part is pi * Gaussian(E2 - E1 - w), utility.py:147-182).
// kubo_pairs:  one CTA per k-point builds the pair records (groups over all bands,
//              degen_thresh; pairs pruned by `nonzero`, dynamic.py:65-69).
// kubo_accum:  one thread per frequency accumulates over the records of a chunk of k-points
//              in shared memory (FP32), then adds the chunk into out (FP64 atomics).
#include <float.h>
#include "wbgpu_common.cuh"
#include "wbgpu_kubo.cuh"

namespace {

__device__ double fermi_dirac(double E, double mu, double kBT) {
  if (kBT == 0.0) return E <= mu ? 1.0 : 0.0;
  if (mu > E + 30 * kBT) return 1.0;
  if (mu < E - 30 * kBT) return 0.0;
  return 1.0 / (exp((E - mu) / kBT) + 1.0);
}

// grid: nk blocks of 128 threads.  Records of k-point k occupy slots [k*P, k*P + count[k]).
template <typename T>
__global__ void kubo_pairs(const double* __restrict__ E, const typename C2<T>::t* __restrict__ Xbar, int nFbar, int iV,
                           int iA, int nw, int external_terms, WbgKubo kp, const double* __restrict__ efermi,
                           double* __restrict__ rec_dE, float* __restrict__ rec_fE, float2* __restrict__ rec_M,
                           int* __restrict__ count, int P) {
  typedef typename C2<T>::t V;
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
  const V* Xk = Xbar + k * nFbar * nw2;
  const double eocc1max = kp.EFmin - 30.0 * kp.kBT, eocc0min = kp.EFmax + 30.0 * kp.kBT;
  for (int pr = threadIdx.x; pr < ng * ng; pr += blockDim.x) {
    const int g1 = pr / ng, g2 = pr % ng;
    if (g1 == g2) continue;  // f_E(E, E) = 0
    const double E1 = Eg[g1], E2 = Eg[g2];
    if ((E1 < eocc1max && E2 < eocc1max) || (E1 > eocc0min && E2 > eocc0min)) continue;
    // M^{ab} = sum_{n in G1, m in G2} i A^a_nm A^b_mn, A = i D + Abar, D_nm = -V_nm / (E_n - E_m)
    V M[9];
    for (int i = 0; i < 9; ++i) M[i] = czero<V>();
    for (int n = gstart[g1]; n < gstart[g1 + 1]; ++n)
      for (int m = gstart[g2]; m < gstart[g2 + 1]; ++m) {
        const double dE = Es[n] - Es[m];
        const T dnm = fabs(dE) < 1e-7 ? T(0) : (T)(1.0 / dE);
        V Anm[3], Amn[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          // i D_nm = -i V_nm / (E_n - E_m);  i D_mn = -i V_mn / (E_m - E_n) = i V_mn / (E_n - E_m)
          Anm[a] = cmuli(cscale(Xk[(iV + a) * nw2 + n * nw + m], -dnm));
          Amn[a] = cmuli(cscale(Xk[(iV + a) * nw2 + m * nw + n], dnm));
          if (external_terms) {
            Anm[a] = cadd(Anm[a], Xk[(iA + a) * nw2 + n * nw + m]);
            Amn[a] = cadd(Amn[a], Xk[(iA + a) * nw2 + m * nw + n]);
          }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) M[3 * a + b] = cadd(M[3 * a + b], cmuli(cmul(Anm[a], Amn[b])));
      }
    const int slot = atomicAdd(&cnt, 1);
    const long long r = k * (long long)P + slot;
    rec_dE[r] = E2 - E1;
    for (int e = 0; e < kp.nEF; ++e)
      rec_fE[r * kp.nEF + e] = (float)(fermi_dirac(E2, efermi[e], kp.kBT) - fermi_dirac(E1, efermi[e], kp.kBT));
    for (int i = 0; i < 9; ++i) rec_M[r * 9 + i] = make_float2((float)M[i].x, (float)M[i].y);
  }
  __syncthreads();
  if (threadIdx.x == 0) count[k] = cnt;
}

// grid: (ceil(nw_freq / TPB), nchunks); out [nEF][nOmega][9] complex128 (accumulated)
__global__ void kubo_accum(const double* __restrict__ rec_dE, const float* __restrict__ rec_fE,
                           const float2* __restrict__ rec_M, const int* __restrict__ count, int P, int nk, int kchunk,
                           const double* __restrict__ omega, WbgKubo kp, double2* __restrict__ out) {
  extern __shared__ float2 acc[];  // [nEF][9][blockDim.x]
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = w < kp.nOmega;
  const int nE = kp.nEF;
  for (int i = 0; i < nE * 9; ++i) acc[i * blockDim.x + threadIdx.x] = make_float2(0.f, 0.f);
  const double om = active ? omega[w] : 0.0;
  const float eta = (float)kp.eta;
  const long long k0 = (long long)blockIdx.y * kchunk;
  const long long k1 = min((long long)nk, k0 + kchunk);
  for (long long k = k0; k < k1; ++k) {
    const int nrec = count[k];
    for (int q = 0; q < nrec; ++q) {
      const long long r = k * (long long)P + q;
      const double dE = rec_dE[r];
      const float delta = (float)(dE - om);  // FP64 difference, FP32 from here on
      const float fd = (float)dE;
      float cre, cim;
      const float den = 1.0f / (delta * delta + eta * eta);
      cre = delta * den;
      cim = eta * den;
      if (kp.gaussian) {
        const float x = delta / eta;
        cim = fabsf(delta) < eta * 14.142135623730951f ? 1.7724538509055160f / eta * expf(-x * x) : 0.0f;
      }
      const float2 fw = make_float2(fd * cre, fd * cim);
      float2 Mv[9];
      for (int i = 0; i < 9; ++i) Mv[i] = rec_M[r * 9 + i];
      for (int e = 0; e < nE; ++e) {
        const float fe = rec_fE[r * nE + e];
        if (fe == 0.0f) continue;
        const float2 c = make_float2(fe * fw.x, fe * fw.y);
        for (int i = 0; i < 9; ++i) {
          float2& a = acc[(e * 9 + i) * blockDim.x + threadIdx.x];
          a.x = fmaf(c.x, Mv[i].x, fmaf(-c.y, Mv[i].y, a.x));
          a.y = fmaf(c.x, Mv[i].y, fmaf(c.y, Mv[i].x, a.y));
        }
      }
    }
  }
  if (!active) return;
  for (int e = 0; e < nE; ++e)
    for (int i = 0; i < 9; ++i) {
      const float2 a = acc[(e * 9 + i) * blockDim.x + threadIdx.x];
      double2* o = out + ((long long)e * kp.nOmega + w) * 9 + i;
      atomicAdd(&o->x, (double)a.x);
      atomicAdd(&o->y, (double)a.y);
    }
}

}  // namespace

size_t wbg_kubo_workspace_bytes(int nw, int nk, int nEF) {
  const size_t P = (size_t)nw * nw;
  return (size_t)nk * P * (8 + 4 * (size_t)nEF + 72) + (size_t)nk * 4 + 1024;
}

int wbg_kubo_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int nw, int nk, int external_terms,
                 const WbgKubo* kp, const double* efermi, const double* omega, void* workspace,
                 size_t workspace_bytes, double* out, int fp64, cudaStream_t stream) {
  if (!E || !Xbar || !kp || !efermi || !omega || !workspace || !out || nw < 1 || nk < 1) return WBG_ERR_ARG;
  if (kp->nEF < 1 || kp->nEF > 64 || kp->nOmega < 1 || !(kp->eta > 0.0)) return WBG_ERR_ARG;
  if (iV < 0 || iV + 3 > nFbar || (external_terms && (iA < 0 || iA + 3 > nFbar))) return WBG_ERR_ARG;
  if (workspace_bytes < wbg_kubo_workspace_bytes(nw, nk, kp->nEF)) return WBG_ERR_WORKSPACE;
  const int P = nw * nw;
  char* w = (char*)workspace;
  double* rec_dE = (double*)w; w += (size_t)nk * P * 8;
  float2* rec_M = (float2*)w; w += (size_t)nk * P * 72;
  float* rec_fE = (float*)w; w += (size_t)nk * P * 4 * kp->nEF;
  int* count = (int*)w;
  const size_t smp = (size_t)nw * 16 + (size_t)(2 * nw + 1) * 4;
  if (fp64)
    kubo_pairs<double><<<nk, 128, smp, stream>>>(E, (const double2*)Xbar, nFbar, iV, iA, nw, external_terms, *kp,
                                                  efermi, rec_dE, rec_fE, rec_M, count, P);
  else
    kubo_pairs<float><<<nk, 128, smp, stream>>>(E, (const float2*)Xbar, nFbar, iV, iA, nw, external_terms, *kp,
                                                 efermi, rec_dE, rec_fE, rec_M, count, P);
  int tpb = 128;
  while (tpb > 32 && (size_t)tpb * kp->nEF * 9 * sizeof(float2) > 96 * 1024) tpb /= 2;
  const size_t sma = (size_t)tpb * kp->nEF * 9 * sizeof(float2);
  if (sma > 220 * 1024) return WBG_ERR_SIZE;
  cudaFuncSetAttribute(kubo_accum, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int wblocks = (kp->nOmega + tpb - 1) / tpb;
  int nchunks = (4 * sms + wblocks - 1) / wblocks;
  if (nchunks > nk) nchunks = nk;
  const int kchunk = (nk + nchunks - 1) / nchunks;
  nchunks = (nk + kchunk - 1) / kchunk;
  kubo_accum<<<dim3(wblocks, nchunks), tpb, sma, stream>>>(rec_dE, rec_fE, rec_M, count, P, nk, kchunk, omega, *kp,
                                                           (double2*)out);
  return wbg_cuda_status(cudaGetLastError());
}
