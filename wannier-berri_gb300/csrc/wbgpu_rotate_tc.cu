// Band-basis rotation Xbar = U^dagger X U on the 5th-generation tensor cores (tcgen05) for
// nw = 32, FP32 path (data_K/data_K.py:130-132 _rotate, data_K/data_K_R.py:69-89 Xbar).
//
// Complex products are embedded in real ones:
//   GEMM1  T = X U       A1[(f,m)][j']  = [Re X_f[m][j] | Im X_f[m][j]]          (K = 2 nw)
//                        B[j'][n']      = [[Re U, Im U], [-Im U, Re U]]          (N = 2 nw)
//                        D1[(f,m)][n']  = [Re T_f[m][n] | Im T_f[m][n]]
//   GEMM2  Y^H = T^H U   A2[(f,m)][j']  = [Re T_f[j][m] | -Im T_f[j][m]]         (same B)
//                        D2[(f,m)][n']  = [Re Y_f^H[m][n] | Im Y_f^H[m][n]]
// so both GEMMs share the embedded U operand, and the fields of one k-point stack along M:
// a 128-row tile holds 4 fields of 32 rows, tiles run over the requested fields.
// Each operand is split as x = hi + lo with hi, lo rounded to TF32 (cvt.rna), and
// A.B = Ah.Bh + (Ah.Bl + Al.Bh) in FP32 (3xTF32, ~2^-21 relative per product).  The tensor
// cores round each accumulation step toward zero, so long chains in one accumulator drift;
// the main products therefore go to NMAIN accumulators over separate K ranges, the small
// correction products to one more, and the partial sums are added on the CUDA cores with
// round-to-nearest -- the result is as accurate as an FP32 CUDA-core GEMM.  Operands live in shared memory in the no-swizzle K-major
// layout: 8-row x 16-byte core matrices, K-adjacent core matrices 144 bytes apart (16 bytes
// of padding) so that the transposed writes of the epilogue hit 32 distinct banks.
// One thread issues the MMAs; completion is tracked with an mbarrier whose every wait is
// bounded in time: on timeout the kernel records WBG_DEVICE_FLAG_TC_TIMEOUT in the
// library's device error word, releases its tensor memory and returns.
#include "wbgpu_common.cuh"
#include "wbgpu_band.cuh"
#include "wbgpu_fixed.cuh"
#include "wbgpu_kubo.cuh"

__device__ unsigned int g_wbg_device_flags;

namespace {

constexpr int NW = 32;                     // Wannier functions handled here
constexpr int KD = 2 * NW;                 // real-embedded contraction length
constexpr int ND = 2 * NW;                 // real-embedded output columns (re | im)
constexpr int TM = 128;                    // MMA M: one tile = 4 fields x 32 rows
constexpr int FPT = TM / NW;               // fields per tile
constexpr int NTHR = 256;                  // warps q and q+4 own TMEM lanes 32q..32q+31 = field q of the tile
constexpr int LBO = 144;                   // bytes between K-adjacent core matrices
constexpr int SBO = (KD / 4) * LBO;        // bytes between 8-row groups
constexpr int A_BYTES = (TM / 8) * SBO;    // one copy (hi or lo) of a tile operand
constexpr int B_BYTES = (ND / 8) * SBO;    // one copy of the embedded U
constexpr int SMEM_BYTES = 2 * B_BYTES + 2 * A_BYTES;
#ifndef WBG_TC_NMAIN
#define WBG_TC_NMAIN 2
#endif
constexpr int NMAIN = WBG_TC_NMAIN;        // accumulators of the main (hi.hi) products
constexpr int NACC = NMAIN + 1;            // + one for the correction products
static_assert((KD / 8) % NMAIN == 0, "K steps must split evenly over the main accumulators");
constexpr uint32_t TMEM_COLS = NACC * ND <= 128 ? 128 : NACC * ND <= 256 ? 256 : 512;  // GEMM1 and GEMM2 share them
constexpr int STAGE_LD = NW + 1;           // float2 row stride of the Hermitian-part staging
// Bound on every mbarrier wait of the kernel: 1 s, settable (wbg_tc_wait_limit) so that a test can
// make a wait run out and exercise the abort path.  After an abort the kernel still waits, for at
// most DRAIN_NS, for the products it has issued, so that no MMA is in flight when its tensor memory
// is freed and the block exits.
__device__ unsigned long long g_tc_wait_ns = 1000000000ull;
constexpr unsigned long long DRAIN_NS = 1000000000ull;
constexpr int TMAP_MAX = 256;              // tile slots (fields + padding) of one launch

static_assert(FPT * NW * STAGE_LD * 8 <= A_BYTES, "staging must fit in the A operand buffer");

// Instruction descriptor of tcgen05.mma kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(ND >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

WBG_D uint32_t op_off(int r, int k) { return (r >> 3) * SBO + (k >> 2) * LBO + (r & 7) * 16 + (k & 3) * 4; }

WBG_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

WBG_D uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// x = hi + lo, both rounded to TF32, stored at byte offset off of the two operand copies
WBG_D void put_split(unsigned char* hi, unsigned char* lo, uint32_t off, float x) {
  const uint32_t h = tf32_rna(x);
  const uint32_t l = tf32_rna(x - __uint_as_float(h));
  *reinterpret_cast<uint32_t*>(hi + off) = h;
  *reinterpret_cast<uint32_t*>(lo + off) = l;
}
// four K-consecutive values (k % 4 == 0: one 16-byte row of a core matrix) in one store each
WBG_D void put_split4(unsigned char* hi, unsigned char* lo, uint32_t off, float a, float b, float c, float d) {
  uint4 h, l;
  h.x = tf32_rna(a);
  h.y = tf32_rna(b);
  h.z = tf32_rna(c);
  h.w = tf32_rna(d);
  l.x = tf32_rna(a - __uint_as_float(h.x));
  l.y = tf32_rna(b - __uint_as_float(h.y));
  l.z = tf32_rna(c - __uint_as_float(h.z));
  l.w = tf32_rna(d - __uint_as_float(h.w));
  *reinterpret_cast<uint4*>(hi + off) = h;
  *reinterpret_cast<uint4*>(lo + off) = l;
}

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), version 1 at bit 46,
// base offset 0, no swizzle.
WBG_D uint64_t make_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(LBO >> 4) << 16) | ((uint64_t)(SBO >> 4) << 32) |
         (1ull << 46);
}

WBG_D void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

WBG_D void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

WBG_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
WBG_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
WBG_D void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// hint: bring the 128-byte line holding p into L2 (no register result, no fault semantics)
WBG_D void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Asynchronous 16-byte global -> shared copies (no registers held, no waits between them)
WBG_D void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
WBG_D void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// The X rows of one tile (FPT fields of NW x NW complex) copied as they are into `raw`
// ([field slot][m][n] float2, FPT * NW * NW * 8 bytes): every copy of the tile is in flight at
// once; slots of padding or of an invalid selection are not copied (the reader fills them).
// Thread `i` of `nthr` takes every nthr-th 16-byte piece.
WBG_D void stage_tile_raw(float2* raw, const float2* X, long long k, int nFin, const int* code, int i, int nthr) {
  constexpr int PIECES = NW * NW / 2;  // 16-byte pieces per field
  for (int c = i; c < FPT * PIECES; c += nthr) {
    const int fl = c / PIECES, pc = c % PIECES;
    const int cd = code[fl];
    if (cd < 0) continue;
    const float2* Xf = X + (k * nFin + (cd & 0x3fffffff)) * (long long)(NW * NW);
    cp_async16(raw + fl * NW * NW + 2 * pc, Xf + 2 * pc);
  }
}

// Elements n0..n0+3 of row m of slot fl from the raw copy: a field given by its lower triangle is
// read as the Hermitian matrix it stands for (X[m][n] = conj(X[n][m]) above the diagonal, real
// diagonal); padding reads 0, an invalid selection NaN.
WBG_D void tile_chunk(const float2* raw, int code, int fl, int m, int n0, float2 (&v)[4]) {
  if (code < 0) {
    const float f = code == -2 ? __int_as_float(0x7fc00000) : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = make_float2(f, f);
    return;
  }
  const bool lower = (code >> 30) != 0;
  const float2* Xf = raw + fl * NW * NW;
  const float4 a = *reinterpret_cast<const float4*>(Xf + m * NW + n0);
  const float4 b = *reinterpret_cast<const float4*>(Xf + m * NW + n0 + 2);
  v[0] = make_float2(a.x, a.y);
  v[1] = make_float2(a.z, a.w);
  v[2] = make_float2(b.x, b.y);
  v[3] = make_float2(b.z, b.w);
  if (lower && m <= n0 + 3) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = n0 + q;
      if (m < n) {
        const float2 w = Xf[n * NW + m];
        v[q] = make_float2(w.x, -w.y);
      } else if (m == n) {
        v[q].y = 0.f;
      }
    }
  }
}

WBG_D unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Phase test of an mbarrier: the potentially blocking try_wait, or (WBG_TC_SPIN) the
// non-blocking test_wait polled in a loop.
#ifndef WBG_TC_SPIN
#define WBG_TC_SPIN 0
#endif
WBG_D bool mbar_poll(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
#if WBG_TC_SPIN
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
#else
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
#endif
  return ok != 0;
}

// Wait for phase `parity` of the mbarrier to complete, for at most limit_ns.
WBG_D bool mbar_wait(uint32_t mbar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (true) {
    if (mbar_poll(mbar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

WBG_D void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// the loaded registers are valid only after tcgen05.wait::ld; passing them through an asm
// after the wait keeps every use behind it
WBG_D void tmem_ld_wait16(uint32_t* r) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
               "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
               "+r"(r[14]), "+r"(r[15])::"memory");
}
// 16 columns (from col) of this thread's TMEM lane, summed over the NACC accumulators
// (correction first, then the main ones) on the CUDA cores with round-to-nearest.
WBG_D void tmem_cols16(uint32_t taddr, int col, float (&v)[16]) {
  uint32_t r[NACC][16];
#pragma unroll
  for (int a = 0; a < NACC; ++a) tmem_ld16(taddr + (uint32_t)(a == 0 ? NMAIN : a - 1) * ND + col, r[a]);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int a = 0; a < NACC; ++a) tmem_ld_wait16(r[a]);
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float x = __uint_as_float(r[0][i]);
#pragma unroll
    for (int a = 1; a < NACC; ++a) x += __uint_as_float(r[a][i]);
    v[i] = x;
  }
}

// Accumulators (ND columns each) from column d: main products of K range q at d + q*ND
// (q < NMAIN), correction products at d + NMAIN*ND.
WBG_D void issue_gemm(uint32_t d, const unsigned char* Ah, const unsigned char* Al, const unsigned char* Bh,
                      const unsigned char* Bl) {
  const uint32_t ah = smem_u32(Ah), al = smem_u32(Al), bh = smem_u32(Bh), bl = smem_u32(Bl);
  constexpr int SPQ = (KD / 8) / NMAIN;  // K steps per main accumulator
#pragma unroll
  for (int s = 0; s < KD / 8; ++s) {  // K = 8 tf32 per instruction = two core matrices
    const uint32_t so = (uint32_t)s * 2 * LBO;
    const uint32_t dm = d + (uint32_t)(s / SPQ) * ND, dc = d + (uint32_t)NMAIN * ND;
    mma_tf32(dc, make_desc(al + so), make_desc(bh + so), s > 0);
    mma_tf32(dc, make_desc(ah + so), make_desc(bl + so), 1);
    mma_tf32(dm, make_desc(ah + so), make_desc(bh + so), s % SPQ != 0);
  }
}

// Every thread waits on the MMA barrier; a timeout anywhere aborts the whole CTA.
WBG_D bool wait_all(uint32_t mbar, uint32_t parity, volatile int* abort_s, unsigned long long limit_ns) {
  if (!mbar_wait(mbar, parity, limit_ns)) {
    *abort_s = 1;
    atomicOr(&g_wbg_device_flags, (unsigned)WBG_DEVICE_FLAG_TC_TIMEOUT);
  }
  __syncthreads();
  return *abort_s == 0;
}

__global__ void __launch_bounds__(NTHR, 2)
    rotate_tc_kernel(const float2* __restrict__ U, long long strideU, const float2* __restrict__ X, int nFin,
                     const int* __restrict__ fsel, const int* __restrict__ herm, int nFrot, float2* __restrict__ Xbar,
                     int nk) {
  extern __shared__ __align__(128) unsigned char smt[];
  unsigned char* Bh = smt;
  unsigned char* Bl = Bh + B_BYTES;
  unsigned char* Ah = Bl + B_BYTES;
  unsigned char* Al = Ah + A_BYTES;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  // tile map: full fields first, then the diagonal-only fields (herm 2); a tile holding only
  // diagonal-only fields stops after T = X U (diag(U^dagger T) by a reduction over the rows)
  __shared__ short tmap_s[TMAP_MAX];
  __shared__ int code_s[TMAP_MAX];
  __shared__ signed char hm_s[TMAP_MAX];
  __shared__ int nfull_s, ntiles_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mb = smem_u32(&mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_s = 0;
    int nf = 0;
    for (int f = 0; f < nFrot; ++f) nf += (herm[f] & 3) != 2;
    const int nt = (nFrot + FPT - 1) / FPT;
    for (int i = 0; i < nt * FPT; ++i) tmap_s[i] = -1;
    int a = 0, b = nf;
    for (int f = 0; f < nFrot; ++f) tmap_s[(herm[f] & 3) == 2 ? b++ : a++] = (short)f;
    // per slot: -1 padding, -2 invalid selection, else source field | lower-triangle input << 30;
    // the output mode herm & 3 (the selection lives in device memory: validated here, once)
    for (int i = 0; i < nt * FPT; ++i) {
      const int f = tmap_s[i];
      int c = -1;
      if (f >= 0) {
        const int fs = fsel[f];
        c = (fs >= 0 && fs < nFin) ? (fs | ((herm[f] & 4) ? (1 << 30) : 0)) : -2;
      }
      code_s[i] = c;
      hm_s[i] = (signed char)(f >= 0 ? (herm[f] & 3) : 0);
    }
    nfull_s = (nf + FPT - 1) / FPT;  // tiles from here on hold diagonal-only fields and padding
    ntiles_s = nt;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base_s;
  const uint32_t D1 = tbase, D2 = tbase;  // GEMM2 reuses GEMM1's accumulators once D1 is read
  const int quarter = warp & 3, half = warp >> 2;  // TMEM lane quarter (= field of the tile), column half
  const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;  // TMEM lanes of this warp
  uint32_t phase = 0;
  const unsigned long long wait_ns = g_tc_wait_ns;
  const int ntiles = ntiles_s, nfull = nfull_s;
  float2* stage = reinterpret_cast<float2*>(Ah) + quarter * NW * STAGE_LD;
  for (long long k = blockIdx.x; k < nk && !abort_s; k += gridDim.x) {
    // ---- embedded U_k (B operand, hi / lo)
    const float2* Uk = U + k * strideU;
    {
      constexpr int PER = NW * NW / NTHR;
      float2 uv[PER];
#pragma unroll
      for (int i = 0; i < PER; ++i) uv[i] = Uk[i * NTHR + tid];  // all loads in flight at once
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int e = i * NTHR + tid, j = e / NW, n = e % NW;
        put_split(Bh, Bl, op_off(n, j), uv[i].x);
        put_split(Bh, Bl, op_off(n, NW + j), -uv[i].y);
        put_split(Bh, Bl, op_off(NW + n, j), uv[i].y);
        put_split(Bh, Bl, op_off(NW + n, NW + j), uv[i].x);
      }
    }
    for (int t = 0; t < ntiles; ++t) {
      // ---- A1: rows (fl, m) of the tile's fields, K = [Re X[m][:] | Im X[m][:]].
      // A task is 4 consecutive elements n0..n0+3 of one row: a 16-byte store per operand half.
      // The tile's rows arrive as a raw copy in the lo half of the operand buffer (all copies in
      // flight at once), every thread takes its chunks from there, then writes hi / lo.
      {
        constexpr int CPR = NW / 4;              // tasks per row
        constexpr int PER = FPT * NW * CPR / NTHR;
        float2* raw = reinterpret_cast<float2*>(Al);
        int code[FPT];  // per field: -1 padding, -2 invalid selection, else source field | lower << 30
#pragma unroll
        for (int fl = 0; fl < FPT; ++fl) code[fl] = code_s[t * FPT + fl];
        stage_tile_raw(raw, X, k, nFin, code, tid, NTHR);
        cp_async_wait_all();
        __syncthreads();
        float2 xv[PER][4];
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int e = i * NTHR + tid, fl = e / (NW * CPR), m = (e / CPR) % NW, n0 = (e % CPR) * 4;
          tile_chunk(raw, code[fl], fl, m, n0, xv[i]);
        }
        __syncthreads();  // the raw copy is read: its space takes the lo operand
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int e = i * NTHR + tid, fl = e / (NW * CPR), m = (e / CPR) % NW, n0 = (e % CPR) * 4;
          const int r = fl * NW + m;
          put_split4(Ah, Al, op_off(r, n0), xv[i][0].x, xv[i][1].x, xv[i][2].x, xv[i][3].x);
          put_split4(Ah, Al, op_off(r, NW + n0), xv[i][0].y, xv[i][1].y, xv[i][2].y, xv[i][3].y);
        }
      }
      fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        issue_gemm(D1, Ah, Al, Bh, Bl);
        mma_commit(mb);
      }
      {  // while the products and the epilogue of this tile run: L2 prefetch of the rows the next
         // tile stages (or of the next k-point's U and first tile)
        const bool last = t + 1 == ntiles;
        const long long kn = last ? k + gridDim.x : k;
        if (kn < nk) {
          const int tn = last ? 0 : t + 1;
          if (last && tid < NW * NW * 8 / 128) prefetch_l2(reinterpret_cast<const char*>(U + kn * strideU) + tid * 128);
          constexpr int CPR = NW / 4;
          constexpr int PER = FPT * NW * CPR / NTHR;
#pragma unroll
          for (int i = 0; i < PER; ++i) {
            const int e = i * NTHR + tid, fl = e / (NW * CPR), m = (e / CPR) % NW, n0 = (e % CPR) * 4;
            if ((n0 & 15) != 0) continue;  // one prefetch per 128-byte line (16 complex floats)
            const int c = code_s[tn * FPT + fl];
            if (c < 0) continue;
            prefetch_l2(X + (kn * nFin + (c & 0x3fffffff)) * (long long)(NW * NW) + m * NW + n0);
          }
        }
      }
      if (!wait_all(mb, phase, &abort_s, wait_ns)) break;
      phase ^= 1;
      tc_fence_after();
      if (t >= nfull) {  // ---- diagonal-only fields: diag_n = Re sum_m conj(U_mn) T_mn
        const int f = tmap_s[t * FPT + quarter];
        float re[16], im[16];
        tmem_cols16(D1 + lane_base, 16 * half, re);  // thread (field q, row m = lane)
        tmem_cols16(D1 + lane_base, NW + 16 * half, im);
        if (f >= 0) {  // warp-uniform
          const float2* Um = U + k * strideU + lane * NW + 16 * half;
          float sum[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const float2 u = Um[i];
            sum[i] = u.x * re[i] + u.y * im[i];
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < 16; ++i) sum[i] += __shfl_xor_sync(0xffffffffu, sum[i], off);
          float v = 0.f;
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (i == lane) v = sum[i];
          if (lane < 16) {
            const int n = 16 * half + lane;
            Xbar[(k * nFrot + f) * (long long)(NW * NW) + n * NW + n] = make_float2(v, 0.f);
          }
        }
        tc_fence_before();
        __syncthreads();  // TMEM columns and the A buffers are reused by the next tile
        continue;
      }
      {  // ---- D1 -> A2: thread (field q, row j) holds T[j][:]; writes column j of T^H.
        // Column half 0 (Re T) -> K block 0, half 1 (Im T) -> K block 1 with a minus sign.
        const int row0 = quarter * NW;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          float v[16];
          tmem_cols16(D1 + lane_base, NW * half + 16 * c, v);
#pragma unroll
          for (int i = 0; i < 16; ++i)
            put_split(Ah, Al, op_off(row0 + 16 * c + i, NW * half + lane), half ? -v[i] : v[i]);
        }
      }
      tc_fence_before();
      fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        issue_gemm(D2, Ah, Al, Bh, Bl);
        mma_commit(mb);
      }
      if (!wait_all(mb, phase, &abort_s, wait_ns)) break;
      phase ^= 1;
      tc_fence_after();
      {  // ---- D2 -> Xbar: thread (field q, row m) holds Y^H[m][n] for n in its column half
        const int f = tmap_s[t * FPT + quarter];
        const int hm = hm_s[t * FPT + quarter];
        float2* dst = Xbar + (k * nFrot + (f >= 0 ? f : 0)) * (long long)(NW * NW);
        float re[16], im[16];
        tmem_cols16(D2 + lane_base, 16 * half, re);
        tmem_cols16(D2 + lane_base, NW + 16 * half, im);
        if (f >= 0) {  // warp-uniform
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int n = 16 * half + i;
            if (hm == 0) dst[n * NW + lane] = make_float2(re[i], -im[i]);  // Y[n][m] = conj(Y^H[m][n])
            else if (hm == 2) { if (n == lane) dst[n * NW + n] = make_float2(re[i], 0.f); }
            else stage[lane * STAGE_LD + n] = make_float2(re[i], im[i]);
          }
        }
        __syncthreads();  // both column halves of every field are staged
        if (f >= 0 && hm == 1) {  // Hermitian part P = (Y^H + Y)/2; P[n][m] = conj(P[m][n])
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int n = 16 * half + i;
            const float2 a = stage[lane * STAGE_LD + n], b = stage[n * STAGE_LD + lane];
            dst[n * NW + lane] = make_float2(0.5f * (a.x + b.x), -0.5f * (a.y - b.y));
          }
        }
      }
      tc_fence_before();
      __syncthreads();  // TMEM columns and the A buffers are reused by the next tile
    }
  }
  if (abort_s) {  // a wait ran out: let the products already issued (phase `phase`) finish first
    if (tid == 0) mbar_wait(mb, phase, DRAIN_NS);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------------------
// Warp-specialised form of the same rotation (one CTA per SM, two tiles in flight):
//   warps 8-11  loaders: the embedded U of the next k-point into B[k % 2] and the X rows of
//               the next tile into A[t % 2] (a raw asynchronous copy, then split into TF32 hi / lo);
//   warp 12     one thread issues, whichever is ready first, GEMM1 (T = X U into TMEM D[t % 2])
//               of the next tile or GEMM2 (Y^H = T^H U into the same columns) of a tile whose
//               T^H is staged;
//   warps 0-7   epilogue: TMEM -> T^H (into A[t % 2], whose X rows GEMM1 has consumed), then
//               TMEM -> Xbar (diagonal-only tiles: diag(U^dagger T) by a row reduction).
// Buffers hand over through mbarriers (one phase per tile and buffer, so the parity of use u
// of a buffer is u & 1); every wait is bounded in time (the abort path of rotate_tc_kernel: a
// collective decision inside each role, the tensor memory freed only after the issued products
// have completed).  While the epilogue turns tile t around, the loaders fill tile t + 1.
// Measured on GB300 (nw = 32, 9 fields, 55 296 k-points): 4.5 ms against 3.9 ms for the
// one-tile-at-a-time kernel with two CTAs per SM; an event trace shows each GEMM of 24
// tcgen05.mma (M = 128, N = 64, K = 8) taking 1.3-1.8 us from issue to completion, so the MMA
// stream of one CTA sets the pace and two CTAs' streams interleave better than one CTA's roles.
// ---------------------------------------------------------------------------------------
#ifndef WBG_TC_TRACE
#define WBG_TC_TRACE 0
#endif
#if WBG_TC_TRACE
// event timeline of CTA 0 (profiling builds only): tag << 56 | tile << 32 | ns since the first event
__device__ unsigned long long g_tc_trace[8192];
__device__ unsigned int g_tc_trace_n;
__device__ unsigned long long g_tc_trace_t0;
WBG_D void tc_trace(int tag, long long tile) {
  if (blockIdx.x != 0 || tile >= 64) return;
  const unsigned int i = atomicAdd(&g_tc_trace_n, 1u);
  if (i < 8192) {
    atomicCAS(&g_tc_trace_t0, 0ull, global_ns());
    g_tc_trace[i] = ((unsigned long long)tag << 56) | ((unsigned long long)tile << 32) |
                    ((global_ns() - g_tc_trace_t0) & 0xffffffffull);
  }
}
#define TC_TRACE(tag, tile) tc_trace(tag, tile)
#else
#define TC_TRACE(tag, tile)
#endif
constexpr int PIPE_EPI = 256;                      // epilogue: warps 0-7
constexpr int PIPE_LD0 = 256, PIPE_LDN = 128;      // loaders: warps 8-11
constexpr int PIPE_MMA_WARP = 12;
constexpr int PIPE_THR = 13 * 32;
constexpr int PIPE_SMEM = 2 * (2 * B_BYTES) + 2 * (2 * A_BYTES);  // B[2] and A[2], hi and lo each
constexpr uint32_t PIPE_TMEM_COLS = 512;           // D[0] at column 0, D[1] at column 256
static_assert(NACC * ND <= 256, "one tile's accumulators must fit 256 TMEM columns");

WBG_D void mbar_init(uint32_t mb) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory"); }
WBG_D void mbar_arrive(uint32_t mb) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mb) : "memory");
}
WBG_D bool mbar_test(uint32_t mb, uint32_t parity) { return mbar_poll(mb, parity); }
// non-blocking phase test (the issue thread polls several barriers in turn)
WBG_D bool mbar_test_nb(uint32_t mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mb), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait that also gives up as soon as another role has aborted
WBG_D bool pipe_wait(uint32_t mb, uint32_t parity, volatile int* abort_s, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (!mbar_test(mb, parity)) {
    if (*abort_s) return false;
    if (global_ns() - t0 > limit_ns) {
      *abort_s = 1;
      atomicOr(&g_wbg_device_flags, (unsigned)WBG_DEVICE_FLAG_TC_TIMEOUT);
      return false;
    }
  }
  return true;
}
WBG_D void named_sync(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
// named barrier with an OR over the participants' predicates: one decision for the whole role
WBG_D bool named_any(int id, int count, bool pred) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
      "selp.s32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((int)pred), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(PIPE_THR, 1)
    rotate_tc_pipe(const float2* __restrict__ U, long long strideU, const float2* __restrict__ X, int nFin,
                   const int* __restrict__ fsel, const int* __restrict__ herm, int nFrot, float2* __restrict__ Xbar,
                   int nk) {
  extern __shared__ __align__(128) unsigned char smp[];
  unsigned char* Bbuf = smp;                     // [2][hi | lo] embedded U
  unsigned char* Abuf = smp + 4 * B_BYTES;       // [2][hi | lo] tile operand (X rows, then T^H)
  __shared__ __align__(8) uint64_t bar_s[14];    // full_b[2] free_b[2] full_a1[2] mma1[2] full_a2[2] mma2[2] free[2]
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  __shared__ short tmap_s[TMAP_MAX];
  __shared__ int code_s[TMAP_MAX];
  __shared__ signed char hm_s[TMAP_MAX];
  __shared__ int nfull_s, ntiles_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto bar = [&](int which, int b) { return smem_u32(&bar_s[2 * which + b]); };
  enum { FULL_B = 0, FREE_B = 1, FULL_A1 = 2, MMA1 = 3, FULL_A2 = 4, MMA2 = 5, FREE_T = 6 };
  if (tid == 0) {
    for (int i = 0; i < 14; ++i) mbar_init(smem_u32(&bar_s[i]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_s = 0;
    int nf = 0;
    for (int f = 0; f < nFrot; ++f) nf += (herm[f] & 3) != 2;
    const int nt = (nFrot + FPT - 1) / FPT;
    for (int i = 0; i < nt * FPT; ++i) tmap_s[i] = -1;
    int a = 0, b = nf;
    for (int f = 0; f < nFrot; ++f) tmap_s[(herm[f] & 3) == 2 ? b++ : a++] = (short)f;
    // per slot: -1 padding, -2 invalid selection, else source field | lower-triangle input << 30;
    // the output mode herm & 3 (the selection lives in device memory: validated here, once)
    for (int i = 0; i < nt * FPT; ++i) {
      const int f = tmap_s[i];
      int c = -1;
      if (f >= 0) {
        const int fs = fsel[f];
        c = (fs >= 0 && fs < nFin) ? (fs | ((herm[f] & 4) ? (1 << 30) : 0)) : -2;
      }
      code_s[i] = c;
      hm_s[i] = (signed char)(f >= 0 ? (herm[f] & 3) : 0);
    }
    nfull_s = (nf + FPT - 1) / FPT;
    ntiles_s = nt;
  }
  if (warp == PIPE_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(PIPE_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base_s;
  const unsigned long long wait_ns = g_tc_wait_ns;
  const int ntiles = ntiles_s, nfull = nfull_s;
  const long long nkc = blockIdx.x < nk ? (nk - 1 - blockIdx.x) / gridDim.x + 1 : 0;  // k-points of this CTA
  const long long ntt = nkc * ntiles;                                               // its tiles
  if (warp >= 8 && warp < 12) {
    // ================= loaders =================
    const int lt = tid - PIPE_LD0;
    long long tt = 0;
    for (long long i = 0; i < nkc; ++i) {
      const long long k = blockIdx.x + i * gridDim.x;
      const int kb = (int)(i & 1);
      unsigned char* Bh = Bbuf + kb * 2 * B_BYTES;
      unsigned char* Bl = Bh + B_BYTES;
      {
        constexpr int PER = NW * NW / PIPE_LDN;
        const float2* Uk = U + k * strideU;
        float2 uv[PER];
#pragma unroll
        for (int q = 0; q < PER; ++q) uv[q] = Uk[q * PIPE_LDN + lt];
        // U_k's loads are in flight: now wait for its buffer (k-point i - 2 done)
        const bool ok = i < 2 || pipe_wait(bar(FREE_B, kb), (uint32_t)(((i >> 1) - 1) & 1), &abort_s, wait_ns);
        if (named_any(1, PIPE_LDN, !ok || abort_s)) break;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          const int e = q * PIPE_LDN + lt, j = e / NW, n = e % NW;
          put_split(Bh, Bl, op_off(n, j), uv[q].x);
          put_split(Bh, Bl, op_off(n, NW + j), -uv[q].y);
          put_split(Bh, Bl, op_off(NW + n, j), uv[q].y);
          put_split(Bh, Bl, op_off(NW + n, NW + j), uv[q].x);
        }
      }
      fence_async_smem();
      named_sync(1, PIPE_LDN);
      if (lt == 0) mbar_arrive(bar(FULL_B, kb));
      bool stop = false;
      for (int t = 0; t < ntiles; ++t, ++tt) {
        const int b = (int)(tt & 1);
        const long long u = tt >> 1;
        unsigned char* Ah = Abuf + b * 2 * A_BYTES;
        unsigned char* Al = Ah + A_BYTES;
        constexpr int CPR = NW / 4;
        constexpr int PER = FPT * NW * CPR / PIPE_LDN;
        int code[FPT];
#pragma unroll
        for (int fl = 0; fl < FPT; ++fl) code[fl] = code_s[t * FPT + fl];
        const bool ok = u < 1 || pipe_wait(bar(FREE_T, b), (uint32_t)((u - 1) & 1), &abort_s, wait_ns);
        if (named_any(1, PIPE_LDN, !ok || abort_s)) { stop = true; break; }
        if (lt == 0) TC_TRACE(2, tt);
        // the tile's rows as a raw copy in the lo half of its buffer, all copies in flight at once
        float2* raw = reinterpret_cast<float2*>(Al);
        stage_tile_raw(raw, X, k, nFin, code, lt, PIPE_LDN);
        cp_async_wait_all();
        named_sync(1, PIPE_LDN);
        if (lt == 0) TC_TRACE(1, tt);
        float2 xv[PER][4];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          const int e = q * PIPE_LDN + lt, fl = e / (NW * CPR), m = (e / CPR) % NW, n0 = (e % CPR) * 4;
          tile_chunk(raw, code[fl], fl, m, n0, xv[q]);
        }
        named_sync(1, PIPE_LDN);  // the raw copy is read: its space takes the lo operand
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          const int e = q * PIPE_LDN + lt, fl = e / (NW * CPR), m = (e / CPR) % NW, n0 = (e % CPR) * 4;
          const int r = fl * NW + m;
          put_split4(Ah, Al, op_off(r, n0), xv[q][0].x, xv[q][1].x, xv[q][2].x, xv[q][3].x);
          put_split4(Ah, Al, op_off(r, NW + n0), xv[q][0].y, xv[q][1].y, xv[q][2].y, xv[q][3].y);
        }
        fence_async_smem();
        named_sync(1, PIPE_LDN);
        if (lt == 0) {
          TC_TRACE(3, tt);
          mbar_arrive(bar(FULL_A1, b));
        }
      }
      if (stop) break;
    }
  } else if (warp == PIPE_MMA_WARP) {
    // ================= MMA issue (one thread) =================
    if (lane == 0) {
      volatile int* ab = &abort_s;
      uint32_t last_bar = 0, last_par = 0;
      long long g1 = 0, g2 = 0;  // next tile for GEMM1, for GEMM2
      unsigned long long t0 = global_ns();
      while (g2 < ntt && !*ab) {
        bool progress = false;
        if (g1 < ntt) {
          const long long i = g1 / ntiles, u = g1 >> 1;
          const int t = (int)(g1 % ntiles), kb = (int)(i & 1), b = (int)(g1 & 1);
          const bool ready = (t != 0 || mbar_test_nb(bar(FULL_B, kb), (uint32_t)((i >> 1) & 1))) &&
                             (u < 1 || mbar_test_nb(bar(FREE_T, b), (uint32_t)((u - 1) & 1))) &&
                             mbar_test_nb(bar(FULL_A1, b), (uint32_t)(u & 1));
          if (ready) {
            tc_fence_after();
            TC_TRACE(4, g1);
            const unsigned char* Ah = Abuf + b * 2 * A_BYTES;
            const unsigned char* Bh = Bbuf + kb * 2 * B_BYTES;
            issue_gemm(tbase + (uint32_t)b * 256, Ah, Ah + A_BYTES, Bh, Bh + B_BYTES);
            mma_commit(bar(MMA1, b));
            last_bar = bar(MMA1, b);
            last_par = (uint32_t)(u & 1);
            ++g1;
            progress = true;
          }
        }
        if (g2 < g1) {
          const long long i = g2 / ntiles, u = g2 >> 1;
          const int t = (int)(g2 % ntiles), kb = (int)(i & 1), b = (int)(g2 & 1);
          if (mbar_test_nb(bar(FULL_A2, b), (uint32_t)(u & 1))) {
            tc_fence_after();
            TC_TRACE(5, g2);
            const unsigned char* Ah = Abuf + b * 2 * A_BYTES;
            const unsigned char* Bh = Bbuf + kb * 2 * B_BYTES;
            if (t < nfull) issue_gemm(tbase + (uint32_t)b * 256, Ah, Ah + A_BYTES, Bh, Bh + B_BYTES);
            mma_commit(bar(MMA2, b));
            last_bar = bar(MMA2, b);
            last_par = (uint32_t)(u & 1);
            if (t == ntiles - 1) mma_commit(bar(FREE_B, kb));
            ++g2;
            progress = true;
          }
        }
        if (progress) {
          t0 = global_ns();
        } else if (global_ns() - t0 > wait_ns) {
          *ab = 1;
          atomicOr(&g_wbg_device_flags, (unsigned)WBG_DEVICE_FLAG_TC_TIMEOUT);
        }
      }
      if (*ab && last_bar) mbar_wait(last_bar, last_par, DRAIN_NS);  // no product in flight at exit
    }
  } else if (warp < 8) {
    // ================= epilogue =================
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lane quarter (= field of the tile), column half
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    for (long long tt = 0; tt < ntt; ++tt) {
      const long long i = tt / ntiles, u = tt >> 1;
      const int t = (int)(tt % ntiles), b = (int)(tt & 1);
      const long long k = blockIdx.x + i * gridDim.x;
      const bool diag = t >= nfull;
      unsigned char* Ah = Abuf + b * 2 * A_BYTES;
      unsigned char* Al = Ah + A_BYTES;
      const uint32_t D = tbase + (uint32_t)b * 256;
      bool ok = pipe_wait(bar(MMA1, b), (uint32_t)(u & 1), &abort_s, wait_ns);
      if (named_any(2, PIPE_EPI, !ok || abort_s)) break;
      if (tid == 0) TC_TRACE(6, tt);
      tc_fence_after();
      const int f = tmap_s[t * FPT + quarter];
      if (diag) {  // diag_n = Re sum_m conj(U_mn) T_mn
        float re[16], im[16];
        tmem_cols16(D + lane_base, 16 * half, re);
        tmem_cols16(D + lane_base, NW + 16 * half, im);
        if (f >= 0) {
          const float2* Um = U + k * strideU + lane * NW + 16 * half;
          float sum[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const float2 uu = Um[q];
            sum[q] = uu.x * re[q] + uu.y * im[q];
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int q = 0; q < 16; ++q) sum[q] += __shfl_xor_sync(0xffffffffu, sum[q], off);
          float v = 0.f;
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (q == lane) v = sum[q];
          if (lane < 16) {
            const int n = 16 * half + lane;
            Xbar[(k * nFrot + f) * (long long)(NW * NW) + n * NW + n] = make_float2(v, 0.f);
          }
        }
      } else {  // T -> A2 = T^H (rows of field q, K blocks Re | -Im)
        const int row0 = quarter * NW;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          float v[16];
          tmem_cols16(D + lane_base, NW * half + 16 * c, v);
#pragma unroll
          for (int q = 0; q < 16; ++q)
            put_split(Ah, Al, op_off(row0 + 16 * c + q, NW * half + lane), half ? -v[q] : v[q]);
        }
      }
      tc_fence_before();
      fence_async_smem();
      named_sync(2, PIPE_EPI);
      if (tid == 0) {
        TC_TRACE(7, tt);
        mbar_arrive(bar(FULL_A2, b));
      }
      ok = pipe_wait(bar(MMA2, b), (uint32_t)(u & 1), &abort_s, wait_ns);
      if (named_any(2, PIPE_EPI, !ok || abort_s)) break;
      if (tid == 0) TC_TRACE(8, tt);
      tc_fence_after();
      if (!diag) {  // Y^H -> Xbar (Hermitian part staged in the tile's A buffer: GEMM2 has read it)
        const int hm = hm_s[t * FPT + quarter];
        float2* dst = Xbar + (k * nFrot + (f >= 0 ? f : 0)) * (long long)(NW * NW);
        float2* stage = reinterpret_cast<float2*>(Ah) + quarter * NW * STAGE_LD;
        float re[16], im[16];
        tmem_cols16(D + lane_base, 16 * half, re);
        tmem_cols16(D + lane_base, NW + 16 * half, im);
        if (f >= 0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int n = 16 * half + q;
            if (hm == 0) dst[n * NW + lane] = make_float2(re[q], -im[q]);
            else if (hm == 2) { if (n == lane) dst[n * NW + n] = make_float2(re[q], 0.f); }
            else stage[lane * STAGE_LD + n] = make_float2(re[q], im[q]);
          }
        }
        named_sync(2, PIPE_EPI);  // both column halves of every field are staged
        if (f >= 0 && hm == 1) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int n = 16 * half + q;
            const float2 a = stage[lane * STAGE_LD + n], bb = stage[n * STAGE_LD + lane];
            dst[n * NW + lane] = make_float2(0.5f * (a.x + bb.x), -0.5f * (a.y - bb.y));
          }
        }
      }
      tc_fence_before();
      named_sync(2, PIPE_EPI);
      if (tid == 0) {
        TC_TRACE(9, tt);
        mbar_arrive(bar(FREE_T, b));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == PIPE_MMA_WARP) {
    __syncwarp();  // lane 0 ran the issue loop alone: reconverge before the warp-wide dealloc
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(PIPE_TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------------------
// Kubo band sums on the tensor cores (mixed path; calculators/dynamic.py:97-98,
//   restot += factor_omega @ (factor_Efermi x M)):
//   out[w][j] += sum_r F[w][r] G[r][j] per k-point,  F = f_w(dE_r), G[r][(e, c)] = f_E[r][e] M[r][c]
// over the pair records of wbgpu_kubo.cu (dE FP64, f_E and M FP32).  Real embedding with two K
// entries per record (Re F, Im F):
//   A[w][2r + p]      = p ? Im F : Re F                                  M = 128 frequencies
//   B[2j + q][2r + p] = [[Re G, -Im G], [Im G, Re G]][q][p]              N = 2 x (<= 104 columns j)
//   D[w][2j + q]      = q ? Im (F G)[w][j] : Re (F G)[w][j]
// F is formed in FP32 from dE - w taken as (dE_hi - w_hi) + (dE_lo - w_lo) (double-float halves:
// the difference to FP32 accuracy without the FP64 pipe).  Operands are split into TF32 hi + lo
// (3xTF32) as in the rotation.  The records of one k-point run in chunks of KT_RC = 8 (K = 16, two
// MMA K-steps, three products each); KT_FILL = 2 consecutive chunks of a k-point go to a fresh TMEM
// accumulator, so no accumulator takes more than twelve truncating steps (at most ~3e-7 relative
// drift toward zero), and the two accumulators alternate, so that the tensor cores fill one while
// the epilogue drains the other.  The epilogue adds each fill with round-to-nearest into
// per-k-point FP32 sums, and adds those to the fixed-point output once per k-point
// (order-independent: the same bits in any grid shape).
// Roles (512 threads x 128 registers, one CTA per SM): warps 0-7 epilogue (TMEM lane quarter =
// warp & 3, column half = warp >> 2: a fill's loads in two batches), adding each drained fill into
// per-k-point FP32 sums in shared memory; warps 8-15 operand producers (two operand stages,
// records copied three chunks ahead; each thread forms four factors of one frequency row), the
// first of which also issues the chunk's MMAs once the producers are done with it.  Every mbarrier
// wait is bounded by the kernel's wait limit, as in the rotation.
// ---------------------------------------------------------------------------------------
constexpr int KT_M = 128, KT_CT = 104, KT_NMAX = 2 * KT_CT, KT_RC = 8, KT_K = 2 * KT_RC, KT_NST = 2;
constexpr int KT_FILL = 2;  // chunks per accumulator fill: <= 12 truncating steps before a drain
constexpr int KT_LBO = 128;                          // K-adjacent core matrices contiguous
constexpr int KT_SBO = (KT_K / 4) * KT_LBO + 16;     // 8-row groups, 16 bytes apart in banks
constexpr int KT_A_BYTES = (KT_M / 8) * KT_SBO;      // one copy (hi or lo) of F
constexpr int KT_B_BYTES = (KT_NMAX / 8) * KT_SBO;   // one copy of the embedded G
constexpr int KT_STAGE = 2 * KT_A_BYTES + 2 * KT_B_BYTES;
// a chunk's records, copied ahead: dE, f_E of the tile's levels (<= KT_EMAX), M (<= KT_NCMAX)
constexpr int KT_EMAX = 16, KT_NCMAX = 27;
constexpr int KT_REC_BYTES = KT_RC * 8 + KT_RC * KT_EMAX * 4 + KT_RC * KT_NCMAX * 8;
constexpr int KT_NREC = 4;  // record buffers: copies run KT_NREC - 1 chunks ahead (cp_async_wait_ahead)
// per-k-point FP32 sums, row = frequency (TMEM lane), KT_ACC_LD floats apart: rows 848 bytes apart
// fall on eight distinct 16-byte bank groups, so a warp's 16-byte accesses are conflict-free
constexpr int KT_ACC_LD = KT_NMAX + 4;
constexpr int KT_ACC_BYTES = KT_M * KT_ACC_LD * 4;
constexpr int KT_SMEM = KT_NST * KT_STAGE + KT_NREC * KT_REC_BYTES + KT_ACC_BYTES;
constexpr int KT_EPI = 256, KT_PROD0 = 256, KT_PRODN = 256, KT_THR = 16 * 32;
constexpr uint32_t KT_TMEM_COLS = 512;               // accumulator of chunk t at column 256 (t & 1)
static_assert(KT_SMEM <= 220 * 1024, "operand stages, records and the sums must fit one CTA's shared memory");
static_assert(KT_ACC_LD % 4 == 0, "16-byte rows of the sums");

WBG_D uint64_t kt_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(KT_LBO >> 4) << 16) | ((uint64_t)(KT_SBO >> 4) << 32) |
         (1ull << 46);
}
WBG_D uint32_t kt_off(int r, int k) {  // byte offset of element (row r, K index k % 4 == 0) of an operand
  return (uint32_t)((r >> 3) * KT_SBO + (k >> 2) * KT_LBO + (r & 7) * 16);
}
WBG_D void kt_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
WBG_D void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
WBG_D void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
WBG_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// every group but the newest KT_NREC - 1 complete (KT_NREC = 4)
WBG_D void cp_async_wait_ahead() { asm volatile("cp.async.wait_group 3;" ::: "memory"); }

// Records r0 .. r0 + rn - 1 of k-point k into a record buffer: dE, f_E of levels e0 .. e0 + ne - 1,
// the NC components of M; thread i of nthr takes every nthr-th 4- or 8-byte piece.
WBG_D void kt_stage_records(unsigned char* rb, const double* rec_dE, const float* rec_fE, const float2* rec_M,
                            long long rbase, int rn, int nEF, int e0, int ne, int NC, int i, int nthr) {
  double* de = reinterpret_cast<double*>(rb);
  float* fe = reinterpret_cast<float*>(rb + KT_RC * 8);
  float2* mm = reinterpret_cast<float2*>(rb + KT_RC * 8 + KT_RC * KT_EMAX * 4);
  for (int p = i; p < rn; p += nthr) cp_async8(de + p, rec_dE + rbase + p);
  for (int p = i; p < rn * ne; p += nthr) {
    const int r = p / ne, e = p - r * ne;
    cp_async4(fe + r * KT_EMAX + e, rec_fE + (rbase + r) * nEF + e0 + e);
  }
  for (int p = i; p < rn * NC; p += nthr) {
    const int r = p / NC, c = p - r * NC;
    cp_async8(mm + r * KT_NCMAX + c, rec_M + (rbase + r) * NC + c);
  }
}

// Bounded wait of the Kubo kernel: mbarrier.try_wait with a suspend-time hint, so that a waiting
// thread sleeps in the barrier unit (up to 20 us per try) instead of spinning; gives up on an abort
// by another role or after limit_ns, recording the timeout like pipe_wait.
WBG_D bool kt_wait(uint32_t mb, uint32_t parity, volatile int* abort_s, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mb), "r"(parity), "r"(20000u)
        : "memory");
    if (ok) return true;
    if (*abort_s) return false;
    if (global_ns() - t0 > limit_ns) {
      *abort_s = 1;
      atomicOr(&g_wbg_device_flags, (unsigned)WBG_DEVICE_FLAG_TC_TIMEOUT);
      return false;
    }
  }
}

// x rounded to TF32 (10-bit mantissa, to nearest, ties away from zero: the result of cvt.rna.tf32.f32
// for finite x) with two integer operations on the full-rate integer pipe
WBG_D uint32_t tf32_rna_int(float x) { return (__float_as_uint(x) + 0x1000u) & 0xffffe000u; }
// four K-consecutive values split as hi + lo (both TF32) into the two operand copies, as put_split4
WBG_D void kt_split4(unsigned char* hi, unsigned char* lo, uint32_t off, float a, float b, float c, float d) {
  uint4 h, l;
  h.x = tf32_rna_int(a);
  h.y = tf32_rna_int(b);
  h.z = tf32_rna_int(c);
  h.w = tf32_rna_int(d);
  l.x = tf32_rna_int(a - __uint_as_float(h.x));
  l.y = tf32_rna_int(b - __uint_as_float(h.y));
  l.z = tf32_rna_int(c - __uint_as_float(h.z));
  l.w = tf32_rna_int(d - __uint_as_float(h.w));
  *reinterpret_cast<uint4*>(hi + off) = h;
  *reinterpret_cast<uint4*>(lo + off) = l;
}

WBG_D void tmem_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
WBG_D void tmem_ld_wait8(uint32_t* r) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
               "+r"(r[7])::"memory");
}

// f_w of one record for frequency w: dE - w and -dE - w from the double-float halves; formula
// WBG_DYN_OPTCOND dE / (dE - w - i eta), WBG_DYN_SHC_SIMPLE (every spin Hall kind)
// 1 / (-dE - w - i eta) / 2, WBG_DYN_SHIFT smear(-dE - w) + smear(dE - w), otherwise
// smear(-dE - w); Lorentzian or Gaussian (the frequency factors of wbgpu_kubo.cu in FP32)
WBG_D float2 kt_factor(int formula, float deh, float del, float wh, float wl, float eta, int gaussian) {
  const float dp = (deh - wh) + (del - wl), dm = (-deh - wh) + (-del - wl);
  if (formula == WBG_DYN_OPTCOND || formula == WBG_DYN_SHC_SIMPLE) {
    const bool opt = formula == WBG_DYN_OPTCOND;
    const float d = opt ? dp : dm;
    const float den = __fdividef(1.0f, fmaf(d, d, eta * eta));
    float cre = d * den, cim = eta * den;
    if (gaussian) {
      const float x = d / eta;
      cim = fabsf(d) < eta * 14.142135623730951f ? 1.7724538509055160f / eta * __expf(-x * x) : 0.0f;
    }
    const float s = opt ? deh + del : 0.5f;
    return make_float2(s * cre, s * cim);
  }
  auto sm = [&](float x) {
    if (gaussian) {
      const float y = x / eta;
      return fabsf(x) < eta * 14.142135623730951f ? 0.5641895835477563f / eta * __expf(-y * y) : 0.0f;
    }
    return 0.3183098861837907f * eta * __fdividef(1.0f, fmaf(x, x, eta * eta));
  };
  float v = sm(dm);
  if (formula == WBG_DYN_SHIFT) v += sm(dp);
  return make_float2(v, 0.0f);
}

__global__ void __launch_bounds__(KT_THR, 1)
    kubo_tc(const double* __restrict__ rec_dE, const float* __restrict__ rec_fE, const float2* __restrict__ rec_M,
            const int* __restrict__ count, int P, int nk, int kchunk, const double* __restrict__ omega, int nOmega,
            int nEF, int NC, int ctile, float eta, int gaussian, int fgroup, wbg_u64* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char smk[];
  __shared__ __align__(8) uint64_t bar_s[KT_NST + 4];  // empty[KT_NST] accfull[2] accfree[2]
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  __shared__ float2 de_s[KT_NST][KT_RC];      // (hi, lo) of the chunk's dE, per stage
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int w0 = blockIdx.x * KT_M, col0 = blockIdx.z * ctile;
  const int ncol = nEF * NC, nct = min(ctile, ncol - col0);  // ctile <= KT_CT
  const int N = (2 * nct + 15) / 16 * 16;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(KT_M >> 4) << 24);
  const long long k0 = (long long)blockIdx.y * kchunk, k1 = min((long long)nk, k0 + kchunk);
  auto bar = [&](int i) { return smem_u32(&bar_s[i]); };
  enum { EMPTY = 0, ACCFULL = KT_NST, ACCFREE = KT_NST + 2 };
  if (tid == 0) {
    for (int i = 0; i < KT_NST + 2; ++i) mbar_init(bar(i));  // one arrival: the MMA commit
    for (int i = 0; i < 2; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar(ACCFREE + i)), "r"(KT_EPI / 32) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_s = 0;
  }
  for (int i = tid; i < KT_SMEM / 16; i += KT_THR)  // padding rows and columns stay zero
    reinterpret_cast<uint4*>(smk)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == KT_PROD0 / 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(KT_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base_s;
  const unsigned long long wait_ns = g_tc_wait_ns;
  volatile int* ab = &abort_s;
  if (warp >= KT_PROD0 / 32) {
    // ================= operand producers =================
    const int pt = tid - KT_PROD0;
    const int prow = pt & (KT_M - 1), phalf = pt / KT_M;  // row of F; records 4 phalf .. 4 phalf + 3
    const int w = w0 + prow;
    const double om = w < nOmega ? omega[w] : 0.0;
    const float wh = (float)om, wl = (float)(om - (double)wh);
    uint32_t last_bar = 0, last_par = 0;  // the issuing thread's last commit
    // the chunk sequence: (k-point, first record) over the CTA's k-points with records
    const int e0 = col0 / NC, ne = (col0 + nct - 1) / NC - e0 + 1;  // the tile's levels (<= KT_EMAX)
    auto skip_empty = [&](long long& kk, int& rr) {
      while (kk < k1 && rr >= count[kk]) {
        ++kk;
        rr = 0;
      }
    };
    auto rbuf = [&](int tt) { return smk + KT_NST * KT_STAGE + (tt % KT_NREC) * KT_REC_BYTES; };
    long long kc = k0, kf;  // the chunk being formed, and the next one to copy
    int rc = 0, rf;
    skip_empty(kc, rc);
    kf = kc;
    rf = rc;
    auto prefetch = [&](int tt) {  // the records of chunk kf / rf into buffer tt, then advance kf / rf
      if (kf < k1) {
        kt_stage_records(rbuf(tt), rec_dE, rec_fE, rec_M, kf * (long long)P + rf, min(KT_RC, count[kf] - rf), nEF,
                         e0, ne, NC, pt, KT_PRODN);
        rf += KT_RC;
        skip_empty(kf, rf);
      }
      cp_async_commit();  // one group per chunk, empty past the last
    };
    for (int tt = 0; tt < KT_NREC - 1; ++tt) prefetch(tt);
    int f = -1;  // fill sequence number
    for (int t = 0; kc < k1; ++t) {
      const int s = (int)(t % KT_NST), rn = min(KT_RC, count[kc] - rc);
      bool ok = true;
      if (lane == 0 && t >= KT_NST)
        ok = kt_wait(bar(EMPTY + s), (uint32_t)((t / KT_NST - 1) & 1), ab, wait_ns);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (named_any(1, KT_PRODN, !ok || *ab)) break;  // one decision for all producers
      unsigned char* Ah = smk + s * KT_STAGE;
      unsigned char* Al = Ah + KT_A_BYTES;
      unsigned char* Bh = Al + KT_A_BYTES;
      unsigned char* Bl = Bh + KT_B_BYTES;
      prefetch(t + KT_NREC - 1);  // KT_NREC - 1 chunks ahead (its buffer held chunk t - 1, now read)
      cp_async_wait_ahead();      // this chunk's records
      named_sync(1, KT_PRODN);
      const unsigned char* rb = rbuf(t);
      const double* rde = reinterpret_cast<const double*>(rb);
      const float* rfe = reinterpret_cast<const float*>(rb + KT_RC * 8);
      const float2* rm = reinterpret_cast<const float2*>(rb + KT_RC * 8 + KT_RC * KT_EMAX * 4);
      if (pt < KT_RC) {
        const double de = pt < rn ? rde[pt] : 0.0;
        const float h = (float)de;
        de_s[s][pt] = make_float2(h, (float)(de - (double)h));
      }
      named_sync(1, KT_PRODN);
      // A: row prow, records (2q, 2q + 1) -> K entries 4q .. 4q + 3, q = 2 phalf, 2 phalf + 1
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        const int q = 2 * phalf + qq;
        float2 f0 = make_float2(0.f, 0.f), f1 = make_float2(0.f, 0.f);
        if (w < nOmega) {
          const float2 a = de_s[s][2 * q], b = de_s[s][2 * q + 1];
          if (2 * q < rn) f0 = kt_factor(fgroup, a.x, a.y, wh, wl, eta, gaussian);
          if (2 * q + 1 < rn) f1 = kt_factor(fgroup, b.x, b.y, wh, wl, eta, gaussian);
        }
        kt_split4(Ah, Al, kt_off(prow, 4 * q), f0.x, f0.y, f1.x, f1.y);
      }
      // B: rows 2j, 2j + 1 for column j of the tile, records (2q, 2q + 1)
#pragma unroll 2
      for (int idx = pt; idx < nct * (KT_RC / 2); idx += KT_PRODN) {
        const int j = idx % nct, q = idx / nct;
        const int col = col0 + j, e = col / NC, c = col - e * NC;
        float2 g[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = 2 * q + h;
          g[h] = make_float2(0.f, 0.f);
          if (r < rn) {
            const float fe = rfe[r * KT_EMAX + e - e0];
            const float2 m = rm[r * KT_NCMAX + c];
            g[h] = make_float2(fe * m.x, fe * m.y);
          }
        }
        kt_split4(Bh, Bl, kt_off(2 * j, 4 * q), g[0].x, -g[0].y, g[1].x, -g[1].y);
        kt_split4(Bh, Bl, kt_off(2 * j + 1, 4 * q), g[0].y, g[0].x, g[1].y, g[1].x);
      }
      fence_async_smem();
      named_sync(1, KT_PRODN);
      // ---- MMA issue (one thread): the chunk's operands are complete; the accumulators are
      // free once the epilogue has drained the previous chunk
      // fills of up to KT_FILL chunks of one k-point per accumulator; the two accumulators alternate
      const int cik = rc / KT_RC;  // chunk of the k-point
      const bool first = cik % KT_FILL == 0, lastc = cik % KT_FILL == KT_FILL - 1 || rc + KT_RC >= count[kc];
      if (first) ++f;
      const int b = f & 1;
      if (pt == 0 && (!first || f < 2 || kt_wait(bar(ACCFREE + b), (uint32_t)((f / 2 - 1) & 1), ab, wait_ns))) {
        tc_fence_after();
        const uint32_t ah = smem_u32(Ah), al = smem_u32(Al), bh = smem_u32(Bh), bl = smem_u32(Bl);
        const uint32_t D = tbase + (uint32_t)(256 * b);
#pragma unroll
        for (int ks = 0; ks < KT_K / 8; ++ks) {
          const uint32_t so = (uint32_t)ks * 2 * KT_LBO;
          kt_mma(D, kt_desc(ah + so), kt_desc(bh + so), idesc, ks > 0 || !first);
          kt_mma(D, kt_desc(al + so), kt_desc(bh + so), idesc, 1);
          kt_mma(D, kt_desc(ah + so), kt_desc(bl + so), idesc, 1);
        }
        mma_commit(bar(EMPTY + s));
        last_bar = bar(EMPTY + s);  // completes once every product issued so far has
        last_par = (uint32_t)((t / KT_NST) & 1);
        if (lastc) mma_commit(bar(ACCFULL + b));
      }
      rc += KT_RC;
      skip_empty(kc, rc);
    }
    cp_async_wait_all();  // no copy in flight at exit
    if (pt == 0 && *ab && last_bar) mbar_wait(last_bar, last_par, DRAIN_NS);  // no product in flight at exit
  } else {
    // ================= epilogue =================
    const int quarter = warp & 3, half = warp >> 2, row = 32 * quarter + lane, w = w0 + row;
    const int nh = N / 2, n8 = nh / 8;  // this warp's columns [half nh, (half + 1) nh), pieces of 8
    const uint32_t D0 = tbase + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(half * nh);
    float* accs = reinterpret_cast<float*>(smk + KT_NST * KT_STAGE + KT_NREC * KT_REC_BYTES) + row * KT_ACC_LD +
                  half * nh;
    wbg_u64* bad = out + 4 * (long long)nEF * nOmega * NC;
    int t = 0;  // fill sequence number
    bool stop = false;
    for (long long k = k0; k < k1 && !stop; ++k) {
      const int nrec = count[k];
      for (int r0 = 0; r0 < nrec; r0 += KT_FILL * KT_RC, ++t) {
        const int b = t & 1;
        bool ok = true;
        if (lane == 0) ok = kt_wait(bar(ACCFULL + b), (uint32_t)((t / 2) & 1), ab, wait_ns);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {  // a warp-wide decision: the epilogue warps share no barrier after this point
          stop = true;
          break;
        }
        tc_fence_after();
        const uint32_t D = D0 + (uint32_t)(256 * b);
        constexpr int PH = (KT_CT / 8 + 1) / 2;  // pieces per batch of loads
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          uint32_t v[PH][8];
#pragma unroll
          for (int p = 0; p < PH; ++p)
            if (h2 * PH + p < n8) tmem_ld8(D + 8 * (h2 * PH + p), v[p]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (h2 == 1) {
            tc_fence_before();
            __syncwarp();  // every lane's loads are complete: one arrival per warp frees the accumulator
            if (lane == 0) mbar_arrive(bar(ACCFREE + b));
          }
#pragma unroll
          for (int p = 0; p < PH; ++p)
            if (h2 * PH + p < n8) {
              tmem_ld_wait8(v[p]);
              float4* a4 = reinterpret_cast<float4*>(accs + 8 * (h2 * PH + p));
              float4 x = a4[0], y = a4[1];
              x.x += __uint_as_float(v[p][0]);
              x.y += __uint_as_float(v[p][1]);
              x.z += __uint_as_float(v[p][2]);
              x.w += __uint_as_float(v[p][3]);
              y.x += __uint_as_float(v[p][4]);
              y.y += __uint_as_float(v[p][5]);
              y.z += __uint_as_float(v[p][6]);
              y.w += __uint_as_float(v[p][7]);
              a4[0] = x;
              a4[1] = y;
            }
        }
      }
      if (!stop && nrec > 0) {  // the k-point's sums into the fixed-point output
        for (int jj = 0; 2 * jj < nh; ++jj) {
          const int j = (half * nh) / 2 + jj;  // complex column of the tile
          const float2 a = reinterpret_cast<const float2*>(accs)[jj];
          reinterpret_cast<float2*>(accs)[jj] = make_float2(0.f, 0.f);
          if (j < nct && w < nOmega) {
            const int col = col0 + j, e = col / NC, c = col - e * NC;
            wbg_u64* o = out + 4 * (((long long)e * nOmega + w) * NC + c);
            fx_add_double(o, (double)a.x, bad);
            fx_add_double(o + 2, (double)a.y, bad);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == KT_PROD0 / 32) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(KT_TMEM_COLS) : "memory");
  }
}

// A wait that runs out by construction: an mbarrier whose phase never completes, waited on with
// the kernel's bound; records WBG_DEVICE_FLAG_TC_TIMEOUT exactly as the rotation does.
__global__ void tc_wait_probe_kernel(int* result) {
  __shared__ __align__(8) uint64_t mbar;
  __shared__ int abort_s;
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_s = 0;
  }
  __syncthreads();
  const bool ok = wait_all(mb, 0, &abort_s, g_tc_wait_ns);  // nothing arrives: phase 0 never completes
  if (threadIdx.x == 0) *result = ok ? 1 : 0;
}

}  // namespace

bool wbg_rotate_tc_supported(int nw, int fp64, int nFrot) {
  return !fp64 && nw == NW && nFrot >= 1 && nFrot <= TMAP_MAX - 2 * FPT;  // the tile map fits its array
}

int wbg_rotate_tc_run(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
                      int nFrot, void* Xbar, int nw, int nk, cudaStream_t stream, bool serial) {
  if (nw != NW || nFrot > TMAP_MAX - 2 * FPT) return WBG_ERR_SIZE;
  if (nk < 1 || nFrot < 1 || !U || !X || !Xbar || !fsel || !herm) return WBG_ERR_ARG;
  int dev = 0, sms = 0;
  if (const cudaError_t e_ = cudaGetDevice(&dev)) return wbg_cuda_status(e_);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return WBG_ERR_CUDA;
  if (!serial) {  // one CTA per SM (its shared memory and tensor memory take the whole SM)
    if (const cudaError_t e_ = cudaFuncSetAttribute(rotate_tc_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, PIPE_SMEM))
      return wbg_cuda_status(e_);
    const long long grid = nk < sms ? nk : sms;
    rotate_tc_pipe<<<(unsigned)grid, PIPE_THR, PIPE_SMEM, stream>>>((const float2*)U, strideU, (const float2*)X, nFin,
                                                                    fsel, herm, nFrot, (float2*)Xbar, nk);
    return wbg_cuda_status(cudaGetLastError());
  }
  if (const cudaError_t e_ = cudaFuncSetAttribute(rotate_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES))
    return wbg_cuda_status(e_);
  const long long grid = nk < 2ll * sms ? nk : 2ll * sms;
  rotate_tc_kernel<<<(unsigned)grid, NTHR, SMEM_BYTES, stream>>>((const float2*)U, strideU, (const float2*)X, nFin,
                                                                fsel, herm, nFrot, (float2*)Xbar, nk);
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_kubo_tc_run(const double* rec_dE, const void* rec_fE, const void* rec_M, const int* count, int P, int nk,
                    const double* omega, int nOmega, int nEF, int NC, double eta, int gaussian, int formula, void* out,
                    cudaStream_t stream) {
  if (!rec_dE || !rec_fE || !rec_M || !count || !omega || !out || nk < 1 || nOmega < 1 || nEF < 1 || NC < 1 ||
      !(eta > 0.0))
    return WBG_ERR_ARG;
  int dev = 0, sms = 0;
  if (const cudaError_t e_ = cudaGetDevice(&dev)) return wbg_cuda_status(e_);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return WBG_ERR_CUDA;
  const int f = formula == WBG_DYN_OPTCOND || formula == WBG_DYN_SHIFT ? formula
                : (formula >= WBG_DYN_SHC_SIMPLE && formula <= WBG_DYN_SHC_RYOO) ? WBG_DYN_SHC_SIMPLE
                                                                                  : WBG_DYN_INJECTION;
  if (NC > KT_NCMAX) return WBG_ERR_ARG;
  const int ncol = nEF * NC;
  // column tiles of <= KT_CT columns spanning <= KT_EMAX levels, balanced
  const int cmax = KT_CT < (KT_EMAX - 1) * NC ? KT_CT : (KT_EMAX - 1) * NC;
  const int gw = (nOmega + KT_M - 1) / KT_M, gc = (ncol + cmax - 1) / cmax;
  const int ctile = (ncol + gc - 1) / gc;
  int gk = sms / (gw * gc);                // one wave of one CTA per SM
  if (gk < 1) gk = 1;
  if (gk > nk) gk = nk;
  const int kc = (nk + gk - 1) / gk;
  gk = (nk + kc - 1) / kc;
  if (const cudaError_t e_ = cudaFuncSetAttribute(kubo_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, KT_SMEM))
    return wbg_cuda_status(e_);
  kubo_tc<<<dim3(gw, gk, gc), KT_THR, KT_SMEM, stream>>>(rec_dE, (const float*)rec_fE, (const float2*)rec_M, count, P,
                                                        nk, kc, omega, nOmega, nEF, NC, ctile, (float)eta, gaussian, f,
                                                        (wbg_u64*)out);
  return wbg_cuda_status(cudaGetLastError());
}

#if WBG_TC_TRACE
extern "C" int wbg_tc_trace_read(unsigned long long* out, unsigned int* n, int clear) {
  if (const cudaError_t e_ = cudaDeviceSynchronize()) return wbg_cuda_status(e_);
  if (const cudaError_t e_ = cudaMemcpyFromSymbol(n, g_tc_trace_n, sizeof(unsigned int))) return wbg_cuda_status(e_);
  const unsigned int m = *n < 8192 ? *n : 8192;
  if (m && cudaMemcpyFromSymbol(out, g_tc_trace, m * sizeof(unsigned long long)) != cudaSuccess) return WBG_ERR_CUDA;
  if (clear) {
    const unsigned int z = 0;
    const unsigned long long z64 = 0;
    cudaMemcpyToSymbol(g_tc_trace_n, &z, sizeof(z));
    cudaMemcpyToSymbol(g_tc_trace_t0, &z64, sizeof(z64));
  }
  return WBG_OK;
}
#endif

int wbg_tc_wait_limit_run(unsigned long long ns) {
  return wbg_cuda_status(cudaMemcpyToSymbol(g_tc_wait_ns, &ns, sizeof(ns)));
}

int wbg_tc_wait_probe_run(int* result, cudaStream_t stream) {
  if (!result) return WBG_ERR_ARG;
  tc_wait_probe_kernel<<<1, 32, 0, stream>>>(result);
  return wbg_cuda_status(cudaGetLastError());
}

int wbg_device_flags_run(unsigned int* flags, int clear) {
  if (!flags) return WBG_ERR_ARG;
  if (const cudaError_t e_ = cudaDeviceSynchronize()) return wbg_cuda_status(e_);
  if (const cudaError_t e_ = cudaMemcpyFromSymbol(flags, g_wbg_device_flags, sizeof(unsigned int))) return wbg_cuda_status(e_);
  if (clear) {
    const unsigned int zero = 0;
    if (const cudaError_t e_ = cudaMemcpyToSymbol(g_wbg_device_flags, &zero, sizeof(unsigned int))) return wbg_cuda_status(e_);
  }
  return WBG_OK;
}
