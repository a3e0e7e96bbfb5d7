// Internal declarations of the R -> k stage (see wbgpu_r2k.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "../../include/wbgpu.h"

typedef wbg_r2k_geom R2KGeom;
typedef wbg_lattice R2KLattice;

// field kinds (x of the int4 field descriptor)
#define R2K_MOM0 0  // (base)               plain transform of base field
#define R2K_DER1 1  // (base, a)            i (R + t_n - t_m)_a
#define R2K_DER2 2  // (base, a, b)         -(R + t_n - t_m)_a (R + t_n - t_m)_b
#define R2K_ROT 3   // (A0 base, g)         curl of the A-derivative, component g
#define R2K_DROT 4  // (A0 base, g, d)      d/dk_d of the curl

size_t wbg_r2k_workspace_bytes(const R2KGeom* g, int order, int nb, int fp64);
int wbg_r2k_run(const void* X, const int* pairStart, const int* r2, const int* sliceStart, const int* pairR1,
                const int* sliceR0, const void* ph0, const void* ph1, const void* ph2, const int4* fdesc,
                const void* wcc, void* workspace, size_t workspace_bytes, void* out, const R2KGeom* g, int order,
                int nF, const R2KLattice* lat, int nb, int fp64, cudaStream_t stream);
