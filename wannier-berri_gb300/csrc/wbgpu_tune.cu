// Launch-shape table of the autotuner (wbgpu/autotune.py measures, this file stores).
// One int per (parameter, variant, nw), 0 = built-in heuristic; read by the launchers of
// wbgpu_eigh.cu and wbgpu_band.cu on every launch, written only through wbg_tune_set with a
// value that wbg_tune_candidates lists for that (parameter, nw, variant).
#include "wbgpu_common.cuh"
#include "wbgpu_eigh.cuh"
#include "wbgpu_tune.cuh"

namespace {
constexpr int kVariants = 6;
int g_tune[WBG_TUNE_NPARAM][kVariants][WBG_EIGH_NMAX + 1];  // zero-initialised: heuristics

bool valid_key(int param, int nw, int variant) {
  return param >= 0 && param < WBG_TUNE_NPARAM && nw >= 1 && nw <= WBG_EIGH_NMAX && variant >= 0 &&
         variant < kVariants;
}

int candidates(int param, int nw, int variant, int* values, int capacity) {
  if (param == WBG_TUNE_KUBO_ENGINE) {  // one setting for every case: variant 0, nw 1
    if (variant != 0 || nw != 1) return 0;
    int count = 0;
    for (int v = 1; v <= 2 && count < capacity; ++v) values[count++] = v;
    return count;
  }
  if (param <= WBG_TUNE_EIGH_VECTORS_GROUP) return wbg_eigh_tune_candidates(param, nw, variant, values, capacity);
  return wbg_rotate_tune_candidates(param, nw, variant, values, capacity);
}
}  // namespace

int wbg_tuned(int param, int variant, int nw) {
  if (!valid_key(param, nw, variant)) return 0;
  return __atomic_load_n(&g_tune[param][variant][nw], __ATOMIC_RELAXED);
}

extern "C" {

int wbg_tune_candidates(int param, int nw, int variant, int* values, int capacity, int* count) {
  if (!valid_key(param, nw, variant) || !count || capacity < 0 || (capacity > 0 && !values))
    return WBG_STATUS_BAD_ARGUMENT;
  *count = candidates(param, nw, variant, values, capacity);
  return WBG_STATUS_OK;
}

int wbg_tune_set(int param, int nw, int variant, int value) {
  if (!valid_key(param, nw, variant) || value < 0) return WBG_STATUS_BAD_ARGUMENT;
  if (value != 0) {
    int vals[32];
    const int n = candidates(param, nw, variant, vals, 32);
    bool ok = false;
    for (int i = 0; i < n && !ok; ++i) ok = vals[i] == value;
    if (!ok) return WBG_STATUS_BAD_ARGUMENT;
  }
  __atomic_store_n(&g_tune[param][variant][nw], value, __ATOMIC_RELAXED);
  return WBG_STATUS_OK;
}

int wbg_tune_get(int param, int nw, int variant, int* value) {
  if (!valid_key(param, nw, variant) || !value) return WBG_STATUS_BAD_ARGUMENT;
  *value = wbg_tuned(param, variant, nw);
  return WBG_STATUS_OK;
}

}  // extern "C"
