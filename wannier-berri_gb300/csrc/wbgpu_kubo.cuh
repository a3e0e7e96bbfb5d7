// Internal declarations of the dynamic (Kubo-type) stage (see wbgpu_kubo.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "../../include/wbgpu.h"

typedef wbg_kubo_params WbgKubo;

size_t wbg_kubo_workspace_bytes(int nw, int nk, int nEF);
int wbg_dynamic_ncomp_impl(int formula);
size_t wbg_dynamic_workspace_bytes(int formula, int nw, int nk, int nEF);
int wbg_dynamic_run(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* fs, int nw, int nk,
                    const WbgKubo* kp, const double* efermi, const double* omega, void* workspace,
                    size_t workspace_bytes, void* out, int fp64, cudaStream_t stream);
int wbg_kubo_run(const double* E, const void* Xbar, int nFbar, int iV, int iA, int nw, int nk, int external_terms,
                 const WbgKubo* kp, const double* efermi, const double* omega, void* workspace,
                 size_t workspace_bytes, void* out, int fp64, cudaStream_t stream);
