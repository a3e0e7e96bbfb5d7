// Band-basis field access of one k-point and the spin-current matrix
// (formula/covariant.py:689-756), shared by the dynamic pair kernel and the static scan kernel.
#pragma once
#include "wbgpu_common.cuh"
#include "../../include/wbgpu.h"

// band-basis fields of one k-point
template <typename T>
struct KBand {
  typedef typename C2<T>::t V;
  const V* X;
  const double* E;
  int nw;
  long long nw2;
  wbg_dynamic_spec f;
  WBG_D V x(int fld, int p, int q) const { return X[fld * nw2 + (long long)p * nw + q]; }
  WBG_D T dinv(int p, int q) const {  // dEig_inv (data_K.py:290-298)
    const double d = E[p] - E[q];
    return fabs(d) < 1e-7 ? T(0) : (T)(1.0 / d);
  }
  WBG_D V D(int a, int p, int q) const { return cscale(x(f.V + a, p, q), -dinv(p, q)); }
  WBG_D V AH(int a, int p, int q) const {
    V r = cmuli(D(a, p, q));
    if (f.external_terms) r = cadd(r, x(f.A + a, p, q));
    return r;
  }
  // principal-value D of the shift current: -V_pq (E_p - E_q) / ((E_p - E_q)^2 + eta^2)
  WBG_D V Dp(int a, int p, int q) const {
    const double d = E[p] - E[q];
    return cscale(x(f.V + a, p, q), (T)(-d / (d * d + f.sc_eta * f.sc_eta)));
  }
};

// J'[p][q][a][s] of the spin current before (J' + J'^dagger) / 2 (formula/covariant.py:721-756),
// component 3 a + s
template <typename T, int F>
WBG_D void spin_current(const KBand<T>& b, int p, int q, typename C2<T>::t* out) {
  typedef typename C2<T>::t V;
  for (int i = 0; i < 9; ++i) out[i] = czero<V>();
  const int nw = b.nw;
  const T Eq = (T)b.E[q];
  for (int l = 0; l < nw; ++l) {
    V Ls[3], Ra[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const V S = b.x(b.f.S + s, p, l);
      if (F == WBG_DYN_SHC_QIAO)  // E_q S - SH, against D: E_q (S D) - (SH D)
        Ls[s] = csub(cscale(S, Eq), b.x(b.f.SH + s, p, l));
      else
        Ls[s] = S;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (F == WBG_DYN_SHC_QIAO) {
        Ra[a] = b.D(a, l, q);
      } else if (F == WBG_DYN_SHC_RYOO) {
        Ra[a] = b.x(b.f.V + a, l, q);
      } else {  // simple: the velocity with the external term i A_lq (E_l - E_q)
        Ra[a] = b.x(b.f.V + a, l, q);
        if (b.f.external_terms) Ra[a] = cadd(Ra[a], cscale(cmuli(b.x(b.f.A + a, l, q)), (T)(b.E[l] - b.E[q])));
      }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int s = 0; s < 3; ++s) cfma(out[3 * a + s], Ls[s], Ra[a]);
  }
  if (F == WBG_DYN_SHC_QIAO) {
    // + delE_q^a S^s_pq + E_q (-i SR) - (-i SHR)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const T va = b.x(b.f.V + a, q, q).x;
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const V t = csub(cscale(b.x(b.f.SR + 3 * a + s, p, q), Eq), b.x(b.f.SHR + 3 * a + s, p, q));
        out[3 * a + s] = cadd(out[3 * a + s], cadd(cscale(b.x(b.f.S + s, p, q), va), cmuli(cscale(t, T(-1)))));
      }
    }
  } else if (F == WBG_DYN_SHC_RYOO) {
    // -i (E_q SA - SHA)
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const V t = csub(cscale(b.x(b.f.SA + i, p, q), Eq), b.x(b.f.SHA + i, p, q));
      out[i] = cadd(out[i], cmuli(cscale(t, T(-1))));
    }
  }
}
