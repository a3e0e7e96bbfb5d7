// Order-independent (bit-reproducible) histogram sums.
//
// A contribution v (double) enters a histogram entry as the 128-bit two's-complement integer
// floor(v * 2^60), kept as two 64-bit words (lo, hi) = value mod 2^64, value >> 64.  Integer
// additions commute, so an entry accumulated by atomics from any number of threads and blocks, in
// any order, over any number of launches, holds the same bits -- the same result alone and in a
// mix of concurrent requests.  Resolution 2^-60 (8.7e-19) absolute per contribution, range
// |sum| < 2^67 (1.5e20).  Non-finite contributions cannot be represented: they are counted in one
// extra word after the entries, and the readers turn every entry of such a histogram into NaN.
//
// Layout of a histogram of n entries: words [2 i] = lo, [2 i + 1] = hi of entry i, word [2 n] =
// count of non-finite contributions; (2 n + 1) * 8 bytes, zero-initialised by the caller.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "wbgpu_common.cuh"

typedef unsigned long long wbg_u64;

// (lo, hi) of floor(v 2^60) for finite v
WBG_D void fx_split(double v, wbg_u64& lo, wbg_u64& hi) {
  const double t = v * 0x1p-4;  // v 2^60 / 2^64: exact scaling
  double h = floor(t);
  double f = (t - h) * 0x1p64;  // fraction in units of 2^-60, exact, in [0, 2^64]
  if (f >= 0x1p64) {             // t - h rounded up to 1 (|t| far below one ulp of 1)
    f = 0.0;
    h += 1.0;
  }
  hi = (wbg_u64)(long long)h;
  lo = (wbg_u64)f;
}

// entry += (lo, hi): the carry of the low word is taken from the value the low word held right
// before this add, so the pair is exact once every add has completed, whatever the interleaving
WBG_D void fx_add(wbg_u64* entry, wbg_u64 lo, wbg_u64 hi) {
  if (lo == 0 && hi == 0) return;
  const wbg_u64 old = atomicAdd(entry, lo);
  const wbg_u64 carry = (old + lo < old) ? 1ull : 0ull;
  if (hi + carry != 0) atomicAdd(entry + 1, hi + carry);
}

// entry += v; a non-finite v is counted in *nonfinite instead
WBG_D void fx_add_double(wbg_u64* entry, double v, wbg_u64* nonfinite) {
  if (v == 0.0) return;
  if (!isfinite(v)) {
    atomicAdd(nonfinite, 1ull);
    return;
  }
  wbg_u64 lo, hi;
  fx_split(v, lo, hi);
  fx_add(entry, lo, hi);
}

// value of an entry as a double: the three parts hi 2^4, (lo >> 32) 2^-28 and (lo & 2^32-1) 2^-60
// are exact doubles (|hi| < 2^53), summed smallest first
WBG_HD double fx_value(wbg_u64 lo, wbg_u64 hi) {
  const double a = (double)(lo & 0xffffffffull) * 0x1p-60;
  const double b = (double)(lo >> 32) * 0x1p-28;
  return (double)(long long)hi * 0x1p4 + (b + a);
}

// a block's shared-memory histogram (n entries + the non-finite count) added to a global one
WBG_D void fx_flush(const wbg_u64* sh, int n, wbg_u64* global) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) fx_add(global + 2 * i, sh[2 * i], sh[2 * i + 1]);
  if (threadIdx.x == 0 && sh[2 * n]) atomicAdd(global + 2 * n, sh[2 * n]);
}

WBG_D void fx_zero(wbg_u64* sh, int n) {
  for (int i = threadIdx.x; i < 2 * n + 1; i += blockDim.x) sh[i] = 0ull;
}

WBG_HD size_t fx_words(size_t n) { return 2 * n + 1; }
