// Internal declarations of the tetrahedron-method kernels (see wbgpu_tetra.cu).
#pragma once
#include <cuda_runtime.h>
#include "../../include/wbgpu.h"

int wbg_tetra_select_run(const double* E, const double* Ec, const int* slot, const int* blocks, int nblocks,
                         const wbg_tetra_grid* g, int nw, double EF0, double EF1, double degen, int sea,
                         signed char* sel, cudaStream_t stream);
int wbg_tetra_accumulate_run(const double* E, const double* Ec, const int* slot, const int* blocks, int nblocks,
                             const wbg_tetra_grid* g, int nw, const signed char* sel, const double* P, int ncomp,
                             const double* EF, int nEF, int der, int ascending, int fp64, void* hist,
                             cudaStream_t stream);
