// Wigner-Seitz replica search of the MDRS setup (system/system_R.py:572-588 do_ws_dist,
// fourier/rvectors.py:57-227): for every distinct Wannier-centre shift s = t_n - t_m (reduced
// coordinates) and every point p of the mp grid, the supercell images R = pts[p] + sup[q]
// whose Cartesian length |(R + s) L| is smallest, ties within tol.  One thread per (s, p),
// FP64 distances (ties are decided at tol ~ 1e-5 A on lengths of tens of A).  The host then
// assigns the matrix element of (m, n, R mod mp) to each image with weight 1/count.
#include "wbgpu_common.cuh"
#include "wbgpu_r2k.cuh"

namespace {

__global__ void ws_replicas_kernel(const double* __restrict__ shifts, int nshift, const int* __restrict__ pts, int npt,
                                   const int* __restrict__ sup, int nsup, R2KLattice lat, double tol, int maxrep,
                                   int* __restrict__ count, int* __restrict__ repq) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nshift * npt) return;
  const int s = (int)(idx / npt), p = (int)(idx % npt);
  double b[3];
  for (int a = 0; a < 3; ++a) b[a] = pts[p * 3 + a] + shifts[s * 3 + a];
  auto dist = [&](int q) {
    double x = 0.0, y = 0.0, z = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double c = b[a] + sup[q * 3 + a];
      x += c * lat.L[a * 3 + 0];
      y += c * lat.L[a * 3 + 1];
      z += c * lat.L[a * 3 + 2];
    }
    return sqrt(x * x + y * y + z * z);
  };
  double dmin = 1e300;
  for (int q = 0; q < nsup; ++q) dmin = fmin(dmin, dist(q));
  int c = 0;
  for (int q = 0; q < nsup; ++q)
    if (fabs(dist(q) - dmin) < tol) {
      if (c < maxrep) repq[idx * maxrep + c] = q;
      ++c;
    }
  count[idx] = c;  // may exceed maxrep: the caller checks and repeats with more room
}

}  // namespace

int wbg_ws_replicas_run(const double* shifts, int nshift, const int* pts, int npt, const int* sup, int nsup,
                        const R2KLattice* lat, double tol, int maxrep, int* count, int* repq, cudaStream_t stream) {
  if (!shifts || !pts || !sup || !lat || !count || !repq || nshift < 1 || npt < 1 || nsup < 1 || maxrep < 1 ||
      !(tol > 0.0))
    return WBG_ERR_ARG;
  const long long n = (long long)nshift * npt;
  ws_replicas_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(shifts, nshift, pts, npt, sup, nsup, *lat, tol,
                                                                      maxrep, count, repq);
  return wbg_cuda_status(cudaGetLastError());
}
