// Tetrahedron method on the regular grid (grid/tetrahedron.py:15-281, TetraWeightsParal;
// corner energies data_K/data_K_R.py:121-141; accumulation calculators/static.py:80-125).
//
// Every k-point of the dense grid (spacing delta = 1/(NKdiv NKFFT) per axis) owns the
// parallelepiped k +- delta/2, cut into 12 tetrahedra (the k-point and one triangle of a face
// diagonal).  The reference evaluates the 8 corner energies of every k-point separately (8 extra
// Hermitian eigensolves per k-point).  Here the corners are the points of the dense grid
// shifted by +delta/2: corner block c (c = 0..NKdiv-1 per axis) is the FFT grid at shift
// (c + 1/2) delta, evaluated once for the whole run (one extra eigensolve per k-point) and kept
// resident in HBM as Ecorner[row][k][n]; corner_slot maps a corner block to its row.
//
// For k-point j of block i, corner s = (sx, sy, sz) (0 = minus side, the reference's
// eCorners[ix, iy, iz] order) is, per axis: s = 1 -> corner block i, index j; s = 0 -> corner
// block i - 1, index j, or for i = 0 corner block NKdiv - 1, index j - 1 (mod NKFFT: H(k) is
// periodic in the reduced coordinates).
#include "wbgpu_common.cuh"
#include "wbgpu_fixed.cuh"
#include "wbgpu_tetra.cuh"

namespace {

// the 12 tetrahedra: k-point + corners (x, y, z); index s = 4 sx + 2 sy + sz; faces in the
// reference's order (iface 0 then 1; faces normal to x, y, z; triangles 00-01-11, 00-10-11).
__constant__ unsigned char kTetra[12][3] = {{0, 1, 3}, {0, 2, 3}, {0, 1, 5}, {0, 4, 5}, {0, 2, 6}, {0, 4, 6},
                                            {4, 5, 7}, {4, 6, 7}, {2, 3, 7}, {2, 6, 7}, {1, 3, 7}, {1, 5, 7}};

// element offset of corner s of batch k-point kk in Ecorner (times nw)
WBG_D long long corner_row(const wbg_tetra_grid& g, const int* __restrict__ blocks, const int* __restrict__ slot,
                           long long kk, int s) {
  const int nk = g.fft[0] * g.fft[1] * g.fft[2];
  const int b = (int)(kk / nk);
  int kl = (int)(kk % nk);
  int gb = blocks[b];
  if (g.per_block) return ((long long)slot[gb] * 8 + s) * nk + kl;
  int i[3], j[3];
  i[2] = gb % g.div[2];
  gb /= g.div[2];
  i[1] = gb % g.div[1];
  i[0] = gb / g.div[1];
  j[2] = kl % g.fft[2];
  kl /= g.fft[2];
  j[1] = kl % g.fft[1];
  j[0] = kl / g.fft[1];
  int c[3], jj[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int plus = (s >> (2 - a)) & 1;
    if (plus || i[a] > 0) {
      c[a] = plus ? i[a] : i[a] - 1;
      jj[a] = j[a];
    } else {
      c[a] = g.div[a] - 1;
      jj[a] = (j[a] + g.fft[a] - 1) % g.fft[a];
    }
  }
  const int row = slot[(c[0] * g.div[1] + c[1]) * g.div[2] + c[2]];
  return (long long)row * nk + (jj[0] * g.fft[1] + jj[1]) * g.fft[2] + jj[2];
}

WBG_D int warp_min_i(int v) { return __reduce_min_sync(0xffffffffu, v); }
WBG_D int warp_max_i(int v) { return __reduce_max_sync(0xffffffffu, v); }

// ---------------------------------------------------------------------------------------
// Band selection (tetrahedron.py:215-262 weights_all_band_groups, Emin = -inf): groups of
// degenerate bands by the k-point energies; a group is in range when its largest corner
// energy reaches EF0 and its smallest reaches EF1; for the Fermi sea (sea != 0) the bands
// [0, bandmax) with bandmax = 1 + the last band whose corners all lie below EF0, capped at the
// first in-range group.  One warp per k-point.  smem: [G][3][nw] doubles + [G][nw] ints.
// ---------------------------------------------------------------------------------------
__global__ void tetra_select_kernel(const double* __restrict__ E, const double* __restrict__ Ec,
                                    const int* __restrict__ slot, const int* __restrict__ blocks, wbg_tetra_grid g,
                                    int nw, long long nkt, double EF0, double EF1, double degen, int sea,
                                    signed char* __restrict__ sel) {
  extern __shared__ double sm[];
  const int G = blockDim.x / 32, w = threadIdx.x / 32, lane = threadIdx.x % 32;
  double* myE = sm + (size_t)w * 3 * nw;
  double* myMin = myE + nw;
  double* myMax = myMin + nw;
  int* myS = reinterpret_cast<int*>(sm + (size_t)G * 3 * nw) + (size_t)w * nw;
  for (long long kk = (long long)blockIdx.x * G + w; kk < nkt; kk += (long long)gridDim.x * G) {
    long long rows[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) rows[s] = corner_row(g, blocks, slot, kk, s) * nw;
    for (int n = lane; n < nw; n += 32) {
      const double e = E[kk * nw + n];
      double lo = e, hi = e;
#pragma unroll
      for (int s = 0; s < 8; ++s) {
        const double x = Ec[rows[s] + n];
        lo = fmin(lo, x);
        hi = fmax(hi, x);
      }
      myE[n] = e;
      myMin[n] = lo;
      myMax[n] = hi;
    }
    __syncwarp();
    for (int n = lane; n < nw; n += 32) myS[n] = (n == 0) || (myE[n] - myE[n - 1] > degen);
    __syncwarp();
    int f0 = nw, below = 0;
    for (int n = lane; n < nw; n += 32) {
      if (myMax[n] < EF0) below = n + 1;
      if (myS[n]) {
        int ge = n + 1;
        while (ge < nw && !myS[ge]) ++ge;
        double gmax = myMax[n], gmin = myMin[n];
        for (int q = n + 1; q < ge; ++q) {
          gmax = fmax(gmax, myMax[q]);
          gmin = fmin(gmin, myMin[q]);
        }
        if (gmax >= EF0 && gmin <= EF1) f0 = min(f0, n);
      }
    }
    f0 = warp_min_i(f0);
    const int bandmax = sea ? min(warp_max_i(below), f0) : 0;
    for (int n = lane; n < nw; n += 32) {
      int gs = n, ge = n + 1;
      while (!myS[gs]) --gs;
      while (ge < nw && !myS[ge]) ++ge;
      double gmax = myMax[gs], gmin = myMin[gs];
      for (int q = gs + 1; q < ge; ++q) {
        gmax = fmax(gmax, myMax[q]);
        gmin = fmin(gmin, myMin[q]);
      }
      signed char v = 0;
      if (n < bandmax) v = 2;
      else if (gmax >= EF0 && gmin <= EF1) v = 1;
      sel[kk * nw + n] = v;
    }
    __syncwarp();
  }
}

// one tetrahedron's corner energies, sorted, pulled 1e-12 apart, with the reciprocals used by
// the weight formulas
struct Tet {
  double e1, e2, e3, e4, r21, r31, r41, r32, r42, r43;
};

WBG_D Tet make_tet(double a, double b, double c, double d) {
  // sort 4 (network)
  double t;
  if (a > b) { t = a; a = b; b = t; }
  if (c > d) { t = c; c = d; d = t; }
  if (a > c) { t = a; a = c; c = t; }
  if (b > d) { t = b; b = d; d = t; }
  if (b > c) { t = b; b = c; c = t; }
  if (b - a < 1e-12) b = a + 1e-12;
  if (c - b < 1e-12) c = b + 1e-12;
  if (d - c < 1e-12) d = c + 1e-12;
  Tet q;
  q.e1 = a; q.e2 = b; q.e3 = c; q.e4 = d;
  q.r21 = 1.0 / (b - a);
  q.r31 = 1.0 / (c - a);
  q.r41 = 1.0 / (d - a);
  q.r32 = 1.0 / (c - b);
  q.r42 = 1.0 / (d - b);
  q.r43 = 1.0 / (d - c);
  return q;
}

// occupation of the linear tetrahedron (der 0, the reference's accurate piecewise form)
WBG_D double tet_occ(const Tet& q, double ef) {
  if (ef >= q.e4) return 1.0;
  if (ef < q.e1) return 0.0;
  if (ef >= q.e3) {
    const double x = q.e4 - ef;
    return 1.0 - (x * q.r41) * (x * q.r42) * (x * q.r43);
  }
  if (ef >= q.e2) {
    const double a13 = (ef - q.e1) * q.r31, a14 = (ef - q.e1) * q.r41;
    const double a23 = (ef - q.e2) * q.r32, a24 = (ef - q.e2) * q.r42;
    return a23 * a24 + a13 * (a14 * (1.0 - a24) + a24 * (1.0 - a23));
  }
  const double x = ef - q.e1;
  return (x * q.r21) * (x * q.r31) * (x * q.r41);
}

// d occupation / d E_F from the reference's expanded cubic in each region (der 1)
WBG_D double tet_dos(const Tet& q, double ef) {
  if (ef >= q.e4 || ef < q.e1) return 0.0;
  const double e1 = q.e1, e2 = q.e2, e3 = q.e3, e4 = q.e4;
  double c1, c2, c3;
  if (ef >= e3) {
    const double d3 = q.r41 * q.r42 * q.r43;
    c1 = 3.0 * e4 * e4 * d3;
    c2 = -3.0 * e4 * d3;
    c3 = d3;
  } else if (ef >= e2) {
    const double d2 = q.r31 * q.r41 * q.r32 * q.r42;
    c1 = (-2.0 * e1 * ((e3 - e2) * (e4 - e2)) + (2.0 * e2 * e4 + e2 * e2) * (e1 - e3) +
          (e1 * e2 + e2 * e3 + e1 * e3) * (e2 - e4)) * d2;
    c2 = (((e3 - e2) * (e4 - e2)) - (e1 - e3) * (2.0 * e2 + e4) - (e3 + e1 + e2) * (e2 - e4)) * d2;
    c3 = d2 * (e1 + e2 - e3 - e4);
  } else {
    const double d1 = q.r21 * q.r31 * q.r41;
    c1 = 3.0 * e1 * e1 * d1;
    c2 = -3.0 * e1 * d1;
    c3 = d1;
  }
  return c1 + ef * (2.0 * c2 + 3.0 * c3 * ef);
}

// ---- FP32 weights (mixed precision) -------------------------------------------------------
// A band's 9 energies are taken relative to its lowest one, eb, as double-float pairs (hi, lo;
// 48-bit significand), so sorting, the gaps and the 1e-12 separation lose nothing; everything
// after is FP32 relative to the tetrahedron's lowest corner e1 (x = E_F - e1), so each factor
// (x / gap) carries ~1e-7 relative error.  The derivative (der 1) is the product rule applied
// to the accurate piecewise form, the same cubic as the reference's expanded polynomial
// without its cancellation.
struct TetF {
  float c_hi, c_lo;                    // e1 - eb
  float g2, g3, g4;                    // e2 - e1, e3 - e1, e4 - e1 (after the separation)
  float r21, r31, r41, r32, r42, r43;  // reciprocals of the gaps
};

WBG_D bool df_less(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

WBG_D TetF make_tetf(float2 a, float2 b, float2 c, float2 d) {
  float2 t;
  if (df_less(b, a)) { t = a; a = b; b = t; }
  if (df_less(d, c)) { t = c; c = d; d = t; }
  if (df_less(c, a)) { t = a; a = c; c = t; }
  if (df_less(d, b)) { t = b; b = d; d = t; }
  if (df_less(c, b)) { t = b; b = c; c = t; }
  const float sep = 1e-12f;
  float d1 = (b.x - a.x) + (b.y - a.y);
  float d2 = (c.x - b.x) + (c.y - b.y);
  float d3 = (d.x - c.x) + (d.y - c.y);
  if (d1 < sep) { d2 -= sep - d1; d1 = sep; }  // e2 = e1 + sep moves e2 up: the next gap shrinks
  if (d2 < sep) { d3 -= sep - d2; d2 = sep; }
  if (d3 < sep) d3 = sep;
  TetF q;
  q.c_hi = a.x;
  q.c_lo = a.y;
  q.g2 = d1;
  q.g3 = d1 + d2;
  q.g4 = d1 + d2 + d3;
  q.r21 = __frcp_rn(d1);
  q.r31 = __frcp_rn(q.g3);
  q.r41 = __frcp_rn(q.g4);
  q.r32 = __frcp_rn(d2);
  q.r42 = __frcp_rn(d2 + d3);
  q.r43 = __frcp_rn(d3);
  return q;
}

WBG_D float tetf_occ(const TetF& q, float x) {
  if (x >= q.g4) return 1.0f;
  if (x < 0.0f) return 0.0f;
  if (x >= q.g3) {
    const float y = q.g4 - x;
    return 1.0f - (y * q.r41) * (y * q.r42) * (y * q.r43);
  }
  if (x >= q.g2) {
    const float x2 = x - q.g2;
    const float a13 = x * q.r31, a14 = x * q.r41, a23 = x2 * q.r32, a24 = x2 * q.r42;
    return a23 * a24 + a13 * (a14 * (1.0f - a24) + a24 * (1.0f - a23));
  }
  return (x * q.r21) * (x * q.r31) * (x * q.r41);
}

WBG_D float tetf_dos(const TetF& q, float x) {
  if (x >= q.g4 || x < 0.0f) return 0.0f;
  if (x >= q.g3) {
    const float y = q.g4 - x;
    return 3.0f * y * y * (q.r41 * q.r42 * q.r43);
  }
  if (x >= q.g2) {
    const float x2 = x - q.g2;
    const float a13 = x * q.r31, a14 = x * q.r41, a23 = x2 * q.r32, a24 = x2 * q.r42;
    const float B = a14 * (1.0f - a24) + a24 * (1.0f - a23);
    const float dB = q.r41 * (1.0f - a24) - a14 * q.r42 + q.r42 * (1.0f - a23) - a24 * q.r32;
    return q.r32 * a24 + a23 * q.r42 + q.r31 * B + a13 * dB;
  }
  return 3.0f * x * x * (q.r21 * q.r31 * q.r41);
}

// s += v, compensated (error-free two-sum into s.y)
WBG_D void two_sum_add(float2& s, float v) {
  const float t = s.x + v;
  const float bp = t - s.x;
  s.y += (s.x - (t - bp)) + (v - bp);
  s.x = t;
}

WBG_D float2 split_df(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// first index i with EF[i] >= x (EF ascending)
WBG_D int lower_bound(const double* __restrict__ EF, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(EF + mid) < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

constexpr int kWin = 32;  // Fermi levels per window chunk (per-lane column of shared memory)
// shared memory per warp: window sums [kWin][32], level offsets [kWin][32] (FP32 weights only),
// band energies [9][32]; 8 bytes each
constexpr int kWarpSmem = (2 * kWin + 9) * 32;

// ---------------------------------------------------------------------------------------
// Weighted accumulation.  Lane n takes band n of its warp's k-point: for sel 1 the band weight
// w(E_F) = (1/12) sum over the 12 tetrahedra, evaluated on the levels between the band's
// smallest and largest corner energy (0 below, 1 (der 0) / 0 (der 1) above); for sel 2 the
// weight is 1 everywhere (the Fermi sea, der 0).  hist gets the contribution P[k][n] w(E_F) in
// difference form -- hist[i] += P (w(i) - w(i-1)) -- so that the cumulative scan of
// wbg_scan_finalize returns sum P w.  F32: weights in FP32 (mixed precision, see TetF); else
// the reference's FP64 arithmetic.  smem: the block's [nEF][nc] histogram when it fits (else
// atomics go to hist directly) + kWarpSmem doubles per warp.
// ---------------------------------------------------------------------------------------
template <bool F32>
__global__ void tetra_accumulate_kernel(const double* __restrict__ E, const double* __restrict__ Ec,
                                        const int* __restrict__ slot, const int* __restrict__ blocks,
                                        wbg_tetra_grid g, int nw, long long nkt, const signed char* __restrict__ sel,
                                        const double* __restrict__ P, int nc, const double* __restrict__ EF, int nEF,
                                        int der, int ascending, int smem_hist, wbg_u64* __restrict__ hist) {
  extern __shared__ double sm[];
  const int G = blockDim.x / 32, w = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nh = nEF * nc;  // fixed-point histogram entries (wbgpu_fixed.cuh)
  wbg_u64* acc = smem_hist ? reinterpret_cast<wbg_u64*>(sm) : hist;
  wbg_u64* bad = acc + 2 * nh;  // count of non-finite contributions
  double* win = sm + (smem_hist ? fx_words(nh) : 0) + (size_t)w * kWarpSmem;
  float2* winf = reinterpret_cast<float2*>(win);            // F32: compensated window sums
  float2* xs = reinterpret_cast<float2*>(win + kWin * 32);  // F32: E_F - eb per level
  double* ek = win + 2 * kWin * 32;                         // [9][32]: corner s at s * 32 + lane
  float2* ekf = reinterpret_cast<float2*>(ek);              // F32: e - eb as (hi, lo)
  if (smem_hist) {
    fx_zero(acc, nh);
    __syncthreads();
  }
  const double wend = der == 0 ? 1.0 : 0.0;
  for (long long kk = (long long)blockIdx.x * G + w; kk < nkt; kk += (long long)gridDim.x * G) {
    for (int n = lane; n < nw; n += 32) {
      const int s = sel[kk * nw + n];
      if (s == 0) continue;
      const double* Pn = P + (kk * nw + n) * nc;
      if (s == 2) {  // Fermi sea: weight 1 at every level
        if (der == 0)
          for (int c = 0; c < nc; ++c) {
            fx_add_double(acc + 2 * c, Pn[c], bad);
          }
        continue;
      }
      double pv[9];  // the band's values in registers; more than 9 components are read from P
      for (int c = 0; c < nc && c < 9; ++c) pv[c] = Pn[c];
      const double e0 = E[kk * nw + n];
      double lo = e0, hi = e0;
      double ev[8];
#pragma unroll
      for (int s8 = 0; s8 < 8; ++s8) {
        ev[s8] = Ec[corner_row(g, blocks, slot, kk, s8) * nw + n];
        lo = fmin(lo, ev[s8]);
        hi = fmax(hi, ev[s8]);
      }
      if constexpr (F32) {
#pragma unroll
        for (int s8 = 0; s8 < 8; ++s8) ekf[s8 * 32 + lane] = split_df(ev[s8] - lo);
        ekf[8 * 32 + lane] = split_df(e0 - lo);
      } else {
#pragma unroll
        for (int s8 = 0; s8 < 8; ++s8) ek[s8 * 32 + lane] = ev[s8];
      }
      // below lo every weight is 0; from i1 on, E_F exceeds every (separated) tetrahedron top
      int i0 = 0, i1 = nEF;
      if (ascending) {
        i0 = lower_bound(EF, nEF, lo);
        i1 = lower_bound(EF, nEF, hi + 4e-12);
      }
      double wprev = 0.0;
      for (int c0 = i0; c0 < i1; c0 += kWin) {
        const int cn = min(kWin, i1 - c0);
        if constexpr (F32) {
          for (int i = 0; i < cn; ++i) {
            winf[i * 32 + lane] = make_float2(0.0f, 0.0f);
            xs[i * 32 + lane] = split_df(__ldg(EF + c0 + i) - lo);
          }
        } else {
          for (int i = 0; i < cn; ++i) win[i * 32 + lane] = 0.0;
        }
#pragma unroll 1
        for (int t = 0; t < 12; ++t) {
          if constexpr (F32) {
            const TetF q = make_tetf(ekf[8 * 32 + lane], ekf[kTetra[t][0] * 32 + lane], ekf[kTetra[t][1] * 32 + lane],
                                     ekf[kTetra[t][2] * 32 + lane]);
            for (int i = 0; i < cn; ++i) {
              const float2 xb = xs[i * 32 + lane];
              const float x = (xb.x - q.c_hi) + (xb.y - q.c_lo);
              two_sum_add(winf[i * 32 + lane], der == 0 ? tetf_occ(q, x) : tetf_dos(q, x));
            }
          } else {
            const Tet q = make_tet(e0, ek[kTetra[t][0] * 32 + lane], ek[kTetra[t][1] * 32 + lane],
                                   ek[kTetra[t][2] * 32 + lane]);
            if (der == 0)
              for (int i = 0; i < cn; ++i) win[i * 32 + lane] += tet_occ(q, __ldg(EF + c0 + i));
            else
              for (int i = 0; i < cn; ++i) win[i * 32 + lane] += tet_dos(q, __ldg(EF + c0 + i));
          }
        }
        for (int i = 0; i < cn; ++i) {
          double wi;
          if constexpr (F32) {
            const float2 v = winf[i * 32 + lane];
            wi = ((double)v.x + (double)v.y) / 12.0;
          } else {
            wi = win[i * 32 + lane] / 12.0;
          }
          const double d = wi - wprev;
          wprev = wi;
          if (d != 0.0)
            for (int c = 0; c < nc; ++c)
              fx_add_double(acc + 2 * ((c0 + i) * nc + c), (nc <= 9 ? pv[c] : Pn[c]) * d, bad);
        }
      }
      if (i1 < nEF && wend != wprev)
        for (int c = 0; c < nc; ++c)
          fx_add_double(acc + 2 * (i1 * nc + c), (nc <= 9 ? pv[c] : Pn[c]) * (wend - wprev), bad);
    }
  }
  if (smem_hist) {
    __syncthreads();
    fx_flush(acc, nh, hist);
  }
}

int grid_cap(int G, long long nkt, int per_sm) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long nblk = (nkt + G - 1) / G;
  const long long cap = (long long)sms * per_sm;
  return (int)(nblk < cap ? nblk : cap);
}

bool grid_ok(const wbg_tetra_grid* g) {
  for (int a = 0; a < 3; ++a)
    if (g->div[a] < 1 || g->fft[a] < 1) return false;
  return g->per_block == 0 || g->per_block == 1;
}

}  // namespace

int wbg_tetra_select_run(const double* E, const double* Ec, const int* slot, const int* blocks, int nblocks,
                         const wbg_tetra_grid* g, int nw, double EF0, double EF1, double degen, int sea,
                         signed char* sel, cudaStream_t stream) {
  if (!E || !Ec || !slot || !blocks || !g || !sel || nblocks < 1 || nw < 1 || !grid_ok(g)) return WBG_ERR_ARG;
  const long long nkt = (long long)nblocks * g->fft[0] * g->fft[1] * g->fft[2];
  const int G = 4;
  const size_t sm = (size_t)G * nw * (3 * 8 + 4);
  if (sm > 220 * 1024) return WBG_ERR_SIZE;
  cudaFuncSetAttribute(tetra_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  tetra_select_kernel<<<grid_cap(G, nkt, 8), 32 * G, sm, stream>>>(E, Ec, slot, blocks, *g, nw, nkt, EF0, EF1, degen,
                                                                   sea, sel);
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_tetra_accumulate_run(const double* E, const double* Ec, const int* slot, const int* blocks, int nblocks,
                             const wbg_tetra_grid* g, int nw, const signed char* sel, const double* P, int ncomp,
                             const double* EF, int nEF, int der, int ascending, int fp64, void* hist,
                             cudaStream_t stream) {
  if (!E || !Ec || !slot || !blocks || !g || !sel || !P || !EF || !hist || nblocks < 1 || nw < 1 || nEF < 1 ||
      !grid_ok(g))
    return WBG_ERR_ARG;
  if (ncomp < 1 || ncomp > 81 || der < 0 || der > 1 || fp64 < 0 || fp64 > 1) return WBG_ERR_ARG;
  const long long nkt = (long long)nblocks * g->fft[0] * g->fft[1] * g->fft[2];
  const int G = 4;
  const size_t wsm = (size_t)G * kWarpSmem * 8;
  const size_t hsm = fx_words((size_t)nEF * ncomp) * 8;
  const int smem_hist = wsm + hsm <= 200 * 1024;
  const size_t sm = wsm + (smem_hist ? hsm : 0);
  const int nblk = grid_cap(G, nkt, 4);
  if (fp64) {
    cudaFuncSetAttribute(tetra_accumulate_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    tetra_accumulate_kernel<false><<<nblk, 32 * G, sm, stream>>>(E, Ec, slot, blocks, *g, nw, nkt, sel, P, ncomp, EF,
                                                                 nEF, der, ascending, smem_hist, (wbg_u64*)hist);
  } else {
    cudaFuncSetAttribute(tetra_accumulate_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    tetra_accumulate_kernel<true><<<nblk, 32 * G, sm, stream>>>(E, Ec, slot, blocks, *g, nw, nkt, sel, P, ncomp, EF,
                                                                nEF, der, ascending, smem_hist, (wbg_u64*)hist);
  }
  return wbg_cuda_status(cudaGetLastError());
}
