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
// The mixed path's 9- and 27-component band sums on the tensor cores (wbgpu_rotate_tc.cu): the pair
// records of wbg_dynamic_run (dE FP64, f_E and M FP32) into the fixed-point output `out`.
int wbg_kubo_tc_run(const double* rec_dE, const void* rec_fE, const void* rec_M, const int* count, int P, int nk,
                    const double* omega, int nOmega, int nEF, int NC, double eta, int gaussian, int formula, void* out,
                    cudaStream_t stream);
