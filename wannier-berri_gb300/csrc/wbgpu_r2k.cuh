// Internal declarations of the R -> k stage (see wbgpu_r2k.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "../../include/wbgpu.h"

typedef wbg_r2k_geom R2KGeom;
typedef wbg_lattice R2KLattice;

// longest run (R-vectors per pair, pairs per slice, slices) one thread keeps in registers
#define WBG_R2K_MAXLEN 32

// field kinds (x of the int4 field descriptor), applied to the R-space matrices
#define R2K_MOM0 0  // (base)               X_R
#define R2K_DER1 1  // (base, a)            i (R + t_n - t_m)_a X_R
#define R2K_DER2 2  // (base, a, b)         -(R + t_n - t_m)_a (R + t_n - t_m)_b X_R
#define R2K_ROT 3   // (A0 base, g)         curl of i (R + t_n - t_m) A_R, component g
#define R2K_DROT 4  // (A0 base, g, d)      i (R + t_n - t_m)_d times that curl

size_t wbg_r2k_workspace_bytes(const R2KGeom* g, int nF, int nb, int prec);
int wbg_r2k_fields_run(const void* XR, int nBase, const int* iRsorted, int nR, int nw, const int4* fdesc, int nF,
                       const double* wcc, const R2KLattice* lat, int prec, void* XF, cudaStream_t stream);
int wbg_r2k_run(const void* XF, int nF, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
                const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, void* workspace,
                size_t workspace_bytes, void* out, const R2KGeom* g, int nb, int prec, const int* cols, int ncols,
                cudaStream_t stream);
int wbg_ws_replicas_run(const double* shifts, int nshift, const int* pts, int npt, const int* sup, int nsup,
                        const R2KLattice* lat, double tol, int maxrep, int* count, int* repq, cudaStream_t stream);
