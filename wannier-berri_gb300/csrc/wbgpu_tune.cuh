// Internal declarations of the autotuner's launch-shape table (see wbgpu_tune.cu).
#pragma once
#include "../../include/wbgpu.h"

// Tuned value of `param` for (variant, nw); 0 when none is set (use the built-in heuristic).
int wbg_tuned(int param, int variant, int nw);
// Values of a parameter that fit the launch limits (wbgpu_eigh.cu / wbgpu_band.cu); returns the count
// written to values[0 .. capacity).
int wbg_eigh_tune_candidates(int param, int nw, int variant, int* values, int capacity);
int wbg_rotate_tune_candidates(int param, int nw, int variant, int* values, int capacity);
