// Internal declarations of the band-basis stages (see wbgpu_band.cu).
#pragma once
#include <cuda_runtime.h>
#include "../../include/wbgpu.h"

typedef wbg_scan WbgScan;

// bands per lane held in registers by the non-additive (Morb) kernel: nw <= 32 * WBG_BAND_MAXPER
#define WBG_BAND_MAXPER 4

bool wbg_rotate_tc_supported(int nw, int fp64, int nFrot);
// serial = true: the one-tile-at-a-time kernel (two CTAs per SM) instead of the warp-specialised one
int wbg_rotate_tc_run(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                      int nFrot, void* Xbar, int nw, int nk, cudaStream_t stream, bool serial = false);
int wbg_device_flags_run(unsigned int* flags, int clear);
int wbg_tc_wait_limit_run(unsigned long long ns);
int wbg_tc_wait_probe_run(int* result, cudaStream_t stream);
int wbg_rotate_run(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                   int nFrot, void* Xbar, int nw, int nk, int fp64, cudaStream_t stream);
int wbg_berry_omega_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                        const WbgScan* sp, int internal_terms, int external_terms, void* hist, int fp64,
                        cudaStream_t stream, double* tab = nullptr, const signed char* sel = nullptr,
                        double* P = nullptr);
// sel / P (all formula kernels): per-band values for the tetrahedron method instead of the
// histogram (wbg_band_values); sp then only supplies degen_thresh.
int wbg_berry_morb_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iB, int iC, int nw,
                       int nk, const WbgScan* sp, int internal_terms, int external_terms, void* hist, int fp64,
                       cudaStream_t stream, const signed char* sel = nullptr, double* P = nullptr);
int wbg_berry_deromega_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iW, int idA,
                           int idO, int nw, int nk, const WbgScan* sp, int internal_terms, int external_terms,
                           void* hist, int fp64, cudaStream_t stream, const signed char* sel = nullptr,
                           double* P = nullptr);
int wbg_berry_product_run(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                          const WbgScan* sp, int sea, void* hist, int fp64, cudaStream_t stream,
                          const signed char* sel = nullptr, double* P = nullptr);
int wbg_scan_finalize_run(const void* hist, int nEF, int ncomp, double scale, double* out, cudaStream_t stream);
int wbg_berry_scan_run(const double* E, const void* Xbar, int nFbar, int iV, int iW, int nw, int nk, const WbgScan* sp,
                       int formula, int sea, void* hist, int fp64, cudaStream_t stream,
                       const signed char* sel = nullptr, double* P = nullptr,
                       const wbg_dynamic_spec* spin = nullptr);
