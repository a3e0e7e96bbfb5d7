// C ABI entry points (declared in include/wbgpu.h).  Thin argument checks around the
// stage launchers; no entry point allocates memory.
#include "wbgpu_common.cuh"
#include "wbgpu_r2k.cuh"
#include "wbgpu_eigh.cuh"
#include "wbgpu_band.cuh"
#include "wbgpu_kubo.cuh"
#include "wbgpu_tetra.cuh"

#include <atomic>

namespace {
std::atomic<int> g_last_cuda_error{0};
}

int wbg_note_cuda_error(cudaError_t e) {
  g_last_cuda_error.store((int)e, std::memory_order_relaxed);
  return WBG_ERR_CUDA;
}

extern "C" {

int wbg_abi_version(void) { return WBG_ABI_VERSION; }

const char* wbg_last_cuda_error_string(void) {
  const int e = g_last_cuda_error.load(std::memory_order_relaxed);
  return e == 0 ? "none" : cudaGetErrorString((cudaError_t)e);
}

const char* wbg_status_string(int status) {
  switch (status) {
    case WBG_STATUS_OK: return "ok";
    case WBG_STATUS_BAD_ARGUMENT: return "bad argument";
    case WBG_STATUS_TOO_LARGE: return "problem size exceeds kernel limits";
    case WBG_STATUS_CUDA_ERROR: return "CUDA error";
    case WBG_STATUS_NO_CONVERGENCE: return "eigensolver did not converge";
    case WBG_STATUS_WORKSPACE_TOO_SMALL: return "workspace too small";
    default: return "unknown status";
  }
}

int wbg_r2k_fields(const void* XR, int nBase, const int* iR, int nR, int nw, const int* field_desc, int nfields,
                   const double* wcc, const wbg_lattice* lat, int prec, void* XF, void* stream) {
  return wbg_r2k_fields_run(XR, nBase, iR, nR, nw, reinterpret_cast<const int4*>(field_desc), nfields, wcc, lat, prec,
                            XF, (cudaStream_t)stream);
}

int wbg_r2k_workspace_size(const wbg_r2k_geom* g, int nfields, int nblocks, int prec, size_t* bytes) {
  if (!g || !bytes || nfields < 1 || nblocks < 1 || prec < 0 || prec > 4) return WBG_STATUS_BAD_ARGUMENT;
  *bytes = wbg_r2k_workspace_bytes(g, nfields, nblocks, prec);
  return WBG_STATUS_OK;
}

int wbg_r2k(const void* XF, int nfields, const int* pair_start, const int* r2, const int* slice_start,
            const int* pair_r1, const int* slice_r0, const void* ph0, const void* ph1, const void* ph2, int nblocks,
            int prec, void* workspace, size_t workspace_bytes, void* fields_out, const wbg_r2k_geom* g,
            void* stream) {
  if (!XF || !pair_start || !r2 || !slice_start || !pair_r1 || !slice_r0 || !ph0 || !ph1 || !ph2 || !workspace ||
      !fields_out || !g)
    return WBG_STATUS_BAD_ARGUMENT;
  return wbg_r2k_run(XF, nfields, pair_start, r2, slice_start, pair_r1, slice_r0, ph0, ph1, ph2, workspace,
                     workspace_bytes, fields_out, g, nblocks, prec, nullptr, 0, (cudaStream_t)stream);
}

int wbg_r2k_columns(const void* XF, int nfields, const int* cols, int ncols, const int* pair_start, const int* r2,
                    const int* slice_start, const int* pair_r1, const int* slice_r0, const void* ph0, const void* ph1,
                    const void* ph2, int nblocks, int prec, void* workspace, size_t workspace_bytes, void* fields_out,
                    const wbg_r2k_geom* g, void* stream) {
  if (!XF || !cols || !pair_start || !r2 || !slice_start || !pair_r1 || !slice_r0 || !ph0 || !ph1 || !ph2 ||
      !workspace || !fields_out || !g)
    return WBG_STATUS_BAD_ARGUMENT;
  return wbg_r2k_run(XF, nfields, pair_start, r2, slice_start, pair_r1, slice_r0, ph0, ph1, ph2, workspace,
                     workspace_bytes, fields_out, g, nblocks, prec, cols, ncols, (cudaStream_t)stream);
}

int wbg_eigh_workspace_size(int nw, int nk, size_t* bytes) {
  if (!bytes || nw < 1 || nw > WBG_EIGH_NMAX || nk < 1) return WBG_STATUS_BAD_ARGUMENT;
  *bytes = wbg_eigh_workspace_bytes(nw, nk);
  return WBG_STATUS_OK;
}

int wbg_eigh_batched(const void* H, long long strideH, int nw, int nk, double* E, void* U, long long strideU,
                     int mode, void* workspace, size_t workspace_bytes, int* errflag, void* stream) {
  return wbg_eigh_run(H, strideH, nw, nk, E, U, strideU, mode, workspace, workspace_bytes, errflag,
                      (cudaStream_t)stream);
}

int wbg_rotate(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
               int nFrot, void* Xbar, int nw, int nk, int fp64, void* stream) {
  return wbg_rotate_run(U, strideU, X, nFin, fsel, herm, nFrot, Xbar, nw, nk, fp64, (cudaStream_t)stream);
}

int wbg_device_flags(unsigned int* flags, int clear) { return wbg_device_flags_run(flags, clear); }

int wbg_tc_wait_limit(unsigned long long ns) { return wbg_tc_wait_limit_run(ns); }

int wbg_tc_wait_probe(int* result, void* stream) { return wbg_tc_wait_probe_run(result, (cudaStream_t)stream); }

int wbg_berry_scan(const double* E, const void* Xbar, int nFbar, int iV, int iW, int nw, int nk, const wbg_scan* scan,
                   int formula, int sea, void* hist, int fp64, void* stream) {
  return wbg_berry_scan_run(E, Xbar, nFbar, iV, iW, nw, nk, scan, formula, sea, hist, fp64, (cudaStream_t)stream);
}

int wbg_ws_replicas(const double* shifts, int nshift, const int* pts, int npt, const int* sup, int nsup,
                    const wbg_lattice* lat, double tol, int maxrep, int* count, int* repq, void* stream) {
  return wbg_ws_replicas_run(shifts, nshift, pts, npt, sup, nsup, lat, tol, maxrep, count, repq,
                             (cudaStream_t)stream);
}

int wbg_berry_tabulate(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                       double degen_thresh, int internal_terms, int external_terms, double* tab, int fp64,
                       void* stream) {
  if (!tab) return WBG_STATUS_BAD_ARGUMENT;
  WbgScan sp;
  sp.EFmin = -1e300;  // every degenerate group is in the window; no sea group
  sp.EFmax = 1e300;
  sp.dEF = 1.0;
  sp.degen_thresh = degen_thresh;
  sp.nEF = 1;
  sp.reserved = 0;
  return wbg_berry_omega_run(E, Xbar, nFbar, iV, iA, iO, nw, nk, &sp, internal_terms, external_terms, nullptr,
                             fp64 ? 1 : 0, (cudaStream_t)stream, tab);
}

int wbg_berry_omega(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                    const wbg_scan* scan, int internal_terms, int external_terms, void* hist, int fp64,
                    void* stream) {
  return wbg_berry_omega_run(E, Xbar, nFbar, iV, iA, iO, nw, nk, scan, internal_terms, external_terms, hist, fp64,
                             (cudaStream_t)stream);
}

int wbg_berry_morb(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iB, int iC, int nw,
                   int nk, const wbg_scan* scan, int internal_terms, int external_terms, void* hist, int fp64,
                   void* stream) {
  return wbg_berry_morb_run(E, Xbar, nFbar, iV, iA, iO, iB, iC, nw, nk, scan, internal_terms, external_terms, hist, fp64,
                            (cudaStream_t)stream);
}

int wbg_berry_deromega(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iW, int idA,
                       int idO, int nw, int nk, const wbg_scan* scan, int internal_terms, int external_terms,
                       void* hist, int fp64, void* stream) {
  return wbg_berry_deromega_run(E, Xbar, nFbar, iV, iA, iO, iW, idA, idO, nw, nk, scan, internal_terms, external_terms,
                                hist, fp64, (cudaStream_t)stream);
}

int wbg_kubo_workspace_size(int nw, int nk, int nEF, size_t* bytes) {
  if (!bytes || nw < 1 || nk < 1 || nEF < 1) return WBG_STATUS_BAD_ARGUMENT;
  *bytes = wbg_kubo_workspace_bytes(nw, nk, nEF);
  return WBG_STATUS_OK;
}

int wbg_kubo(const double* E, const void* Xbar, int nFbar, int iV, int iA, int nw, int nk, int external_terms,
             const wbg_kubo_params* params, const double* efermi, const double* omega, void* workspace,
             size_t workspace_bytes, void* out, int fp64, void* stream) {
  return wbg_kubo_run(E, Xbar, nFbar, iV, iA, nw, nk, external_terms, params, efermi, omega, workspace,
                      workspace_bytes, out, fp64, (cudaStream_t)stream);
}

int wbg_berry_shc(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* spin, int nw, int nk,
                  const wbg_scan* scan, void* hist, int fp64, void* stream) {
  if (!spin) return WBG_STATUS_BAD_ARGUMENT;
  return wbg_berry_scan_run(E, Xbar, nFbar, spin->V, -1, nw, nk, scan, WBG_FORMULA_SPIN_OMEGA, 1, hist, fp64,
                            (cudaStream_t)stream, nullptr, nullptr, spin);
}

int wbg_dynamic_ncomp(int formula) { return ::wbg_dynamic_ncomp_impl(formula); }

int wbg_dynamic_workspace_size(int formula, int nw, int nk, int nEF, size_t* bytes) {
  if (!bytes || nw < 1 || nk < 1 || nEF < 1 || wbg_dynamic_ncomp(formula) == 0) return WBG_STATUS_BAD_ARGUMENT;
  *bytes = wbg_dynamic_workspace_bytes(formula, nw, nk, nEF);
  return WBG_STATUS_OK;
}

int wbg_dynamic(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* spec, int nw, int nk,
                const wbg_kubo_params* params, const double* efermi, const double* omega, void* workspace,
                size_t workspace_bytes, void* out, int fp64, void* stream) {
  return wbg_dynamic_run(E, Xbar, nFbar, spec, nw, nk, params, efermi, omega, workspace, workspace_bytes, out, fp64,
                         (cudaStream_t)stream);
}

int wbg_tetra_select(const double* E, const double* Ecorner, const int* corner_slot, const int* blocks, int nblocks,
                     const wbg_tetra_grid* grid, int nw, double EF0, double EF1, double degen_thresh, int sea,
                     signed char* sel, void* stream) {
  return wbg_tetra_select_run(E, Ecorner, corner_slot, blocks, nblocks, grid, nw, EF0, EF1, degen_thresh, sea, sel,
                              (cudaStream_t)stream);
}

int wbg_band_values(const double* E, const void* Xbar, int nFbar, const wbg_field_index* f, int nw, int nk,
                    int formula, int internal_terms, int external_terms, double degen_thresh,
                    const signed char* sel, double* P, int fp64, void* stream) {
  if (!f || !sel || !P || (fp64 != 0 && fp64 != 1)) return WBG_STATUS_BAD_ARGUMENT;
  WbgScan sp;
  sp.EFmin = 0.0;  // groups come from sel; no histogram
  sp.EFmax = 0.0;
  sp.dEF = 1.0;
  sp.degen_thresh = degen_thresh;
  sp.nEF = 0;
  sp.reserved = 0;
  cudaStream_t st = (cudaStream_t)stream;
  switch (formula) {
    case WBG_FORMULA_IDENTITY:
    case WBG_FORMULA_INVMASS:
    case WBG_FORMULA_VELVEL:
    case WBG_FORMULA_DIAG:
    case WBG_FORMULA_VELVELVEL:
      return wbg_berry_scan_run(E, Xbar, nFbar, f->V, f->W, nw, nk, &sp, formula, 0, nullptr, fp64, st, sel, P);
    case WBG_FORMULA_OMEGA:
      return wbg_berry_omega_run(E, Xbar, nFbar, f->V, f->A, f->O, nw, nk, &sp, internal_terms, external_terms,
                                 nullptr, fp64, st, nullptr, sel, P);
    case WBG_FORMULA_DEROMEGA:
      return wbg_berry_deromega_run(E, Xbar, nFbar, f->V, f->A, f->O, f->W, f->dA, f->dO, nw, nk, &sp, internal_terms,
                                    external_terms, nullptr, fp64, st, sel, P);
    case WBG_FORMULA_MORB:
      return wbg_berry_morb_run(E, Xbar, nFbar, f->V, f->A, f->O, f->B, f->C, nw, nk, &sp, internal_terms,
                                external_terms, nullptr, fp64, st, sel, P);
    default:
      return WBG_STATUS_BAD_ARGUMENT;
  }
}

int wbg_berry_product(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                      const wbg_scan* scan, int sea, void* hist, int fp64, void* stream) {
  return wbg_berry_product_run(E, Xbar, nFbar, spec, nw, nk, scan, sea, hist, fp64, (cudaStream_t)stream);
}

int wbg_product_values(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                       double degen_thresh, const signed char* sel, double* P, int fp64, void* stream) {
  if (!sel || !P) return WBG_STATUS_BAD_ARGUMENT;
  WbgScan sp;
  sp.EFmin = 0.0;  // groups come from sel; no histogram
  sp.EFmax = 0.0;
  sp.dEF = 1.0;
  sp.degen_thresh = degen_thresh;
  sp.nEF = 0;
  sp.reserved = 0;
  return wbg_berry_product_run(E, Xbar, nFbar, spec, nw, nk, &sp, 0, nullptr, fp64, (cudaStream_t)stream, sel, P);
}

int wbg_tetra_accumulate(const double* E, const double* Ecorner, const int* corner_slot, const int* blocks,
                         int nblocks, const wbg_tetra_grid* grid, int nw, const signed char* sel, const double* P,
                         int ncomp, const double* efermi, int nEF, int der, int ascending, int fp64,
                         void* hist, void* stream) {
  return wbg_tetra_accumulate_run(E, Ecorner, corner_slot, blocks, nblocks, grid, nw, sel, P, ncomp, efermi, nEF, der,
                                  ascending, fp64, hist, (cudaStream_t)stream);
}

int wbg_scan_finalize(const void* hist, int nEF, int ncomp, double scale, double* out, void* stream) {
  return wbg_scan_finalize_run(hist, nEF, ncomp, scale, out, (cudaStream_t)stream);
}

}  // extern "C"
