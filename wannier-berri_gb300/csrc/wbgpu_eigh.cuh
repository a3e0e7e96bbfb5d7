// Internal declarations of the eigensolver stage (see wbgpu_eigh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#define WBG_EIGH_NMAX 128
#include "../../include/wbgpu.h"

size_t wbg_eigh_workspace_bytes(int n, int nk);
int wbg_eigh_run(const void* H, long long strideH, int n, int nk, void* E, void* U, long long strideU,
                 int mode, void* workspace, size_t workspace_bytes, int* errflag, cudaStream_t stream);
