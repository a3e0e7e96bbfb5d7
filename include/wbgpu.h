/*
 * wbgpu -- C ABI of the GB300 (sm_103a) Wannier-interpolation backend.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream (as void*),
 * launches stream-ordered work and returns an int status (WBG_STATUS_*).  No entry point
 * allocates device memory: the caller passes every output and a workspace whose size
 * the matching *_workspace_size query reports.  Complex numbers are interleaved
 * (re, im) pairs of double (fp64 != 0) or float (fp64 == 0); matrices are row-major
 * [m][n] with m, n Wannier indices.
 *
 * Reference interfaces replaced (paths relative to the wannier-berri project root):
 *   wbg_r2k            fourier/fft.py:133-192 FFT_R_to_k.__call__ with
 *                      fourier/rvectors.py:477-506 apply_expdK / derivative / R_to_k and
 *                      data_K/data_K_R.py:28-51,91-97 get_R_mat / rotAA / _R_to_k_H
 *   wbg_eigh_batched   data_K/data_K.py:211-218 E_K / UU_K (np.linalg.eigh of HH_K)
 *   wbg_rotate         data_K/data_K.py:130-132 _rotate and data_K/data_K_R.py:69-89 Xbar
 *   wbg_berry_omega    formula/covariant.py:161-203 Omega traced over the band groups of
 *                      data_K/data_K.py:172-198 and binned as in calculators/static.py:103-136
 *   wbg_scan_finalize  calculators/static.py:131-155 (cumulative Fermi scan, /V /nk * factor)
 */
#ifndef WBGPU_H
#define WBGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WBG_ABI_VERSION 1

#define WBG_STATUS_OK 0
#define WBG_STATUS_BAD_ARGUMENT 1
#define WBG_STATUS_TOO_LARGE 2
#define WBG_STATUS_CUDA_ERROR 3
#define WBG_STATUS_NO_CONVERGENCE 4
#define WBG_STATUS_WORKSPACE_TOO_SMALL 5

/* Geometry of one R -> k transform launch.  R-vectors are sorted by (R0, R1, R2);
 * a "pair" is a run of equal (R0, R1), a "slice" a run of pairs with equal R0. */
typedef struct {
  int nR, nw, nw2, nBase; /* R-vectors, Wannier functions, nw*nw, base fields in XR      */
  int nP, nU;             /* number of (R0,R1) pairs and of R0 slices                    */
  int N0, N1, N2, nk;     /* FFT block grid and nk = N0*N1*N2                            */
  int nr0, nr1, nr2;      /* widths of the per-axis phase tables                         */
  int rmin0, rmin1, rmin2;/* smallest R component per axis (phase table offset)          */
  int maxPairLen, maxSliceLen;
} wbg_r2k_geom;

/* Real lattice, rows are lattice vectors (Angstrom): R_cart = iR . L */
typedef struct {
  double L[9];
} wbg_lattice;

/* Fermi-level scan (calculators/static.py:53-58): levels EFmin + i*dEF, i < nEF */
typedef struct {
  double EFmin, EFmax, dEF, degen_thresh;
  int nEF;
  int reserved;
} wbg_scan;

int wbg_abi_version(void);
const char* wbg_status_string(int status);
/* The CUDA runtime's message for the error behind the most recent WBG_STATUS_CUDA_ERROR that any
 * entry point returned in this process ("none" if there was none); no reference counterpart. */
const char* wbg_last_cuda_error_string(void);

/* ---- stage 1: R -> k --------------------------------------------------------------------
 * wbg_r2k_fields (once per system and field set): R-space arrays of the k-space fields,
 *   XR       [nBase][nR][nw][nw] complex128 base matrices (Ham, then A x/y/z, ...), R sorted
 *   iR       [nR][3] int, the sorted R-vectors;  wcc [nw][3] Cartesian Wannier centres t
 *   field_desc [nfields][4] int (kind, base, a, b): 0 X; 1 i w_a X; 2 -w_a w_b X;
 *            3 curl component a of i w A (A = bases base..base+2); 4 i w_b times that curl,
 *            with w = R + t_n - t_m in Cartesian coordinates (fourier/rvectors.py:355-369,
 *            487-494; data_K/data_K_R.py:48-51)
 *   XF       [nfields][nR][nw][nw] complex: prec 0 float, 1 double, 2 double-float (re.hi, re.lo,
 *            im.hi, im.lo floats: 48-bit significand on the FP32 pipe); prec 3 float followed by
 *            a second [nfields][nR][nw][nw] float array of the rounding residuals XF - float(XF)
 * wbg_r2k (per batch of FFT blocks): fields_out[b*nk + k][f] = sum_R exp(2 pi i R.(j_k/N + dK_b)) XF[f][R]
 *   pair_start [nP+1] first sorted R of each pair;  r2 [nR] third R component
 *   slice_start [nU+1] first pair of each slice;    pair_r1 [nP];  slice_r0 [nU]
 *   ph0/ph1/ph2 [nblocks][N_d][nr_d] complex (precision prec): exp(2 pi i R_d (j/N_d + dK_d)),
 *            R_d = rmin_d + r
 *   fields_out [nblocks*nk][nfields][nw][nw] complex (precision prec), k = (j0*N1 + j1)*N2 + j2
 *   prec 4 (double-float transform stored as complex64): XF, phases and workspace as prec 2,
 *            fields_out complex64 -- each element rounded once from its double-float value.
 *   prec 3 (FP32 with split inputs): the first contraction also sums the residuals of XF, so
 *            the k-independent R-space data -- whose rounding would be a systematic error of the
 *            whole integral -- enter with 48 bits; phases, intermediates and output as prec 0.
 */
int wbg_r2k_fields(const void* XR, int nBase, const int* iR, int nR, int nw, const int* field_desc, int nfields,
                   const double* wcc, const wbg_lattice* lat, int prec, void* XF, void* stream);
int wbg_r2k_workspace_size(const wbg_r2k_geom* g, int nfields, int nblocks, int prec, size_t* bytes);
/* MDRS replica search (system/system_R.py:572-588 do_ws_dist, fourier/rvectors.py:57-227):
 * for every shift s (shifts [nshift][3], reduced t_n - t_m) and grid point p (pts [npt][3],
 * the mp grid), the images R = pts[p] + sup[q] (sup [nsup][3], supercell offsets) with the
 * smallest |(R + s) L|, ties within tol: count [nshift][npt], and the first maxrep image
 * indices q in repq [nshift][npt][maxrep] (count > maxrep: repeat with more room).  Setup
 * step, once per system; all pointers on the device. */
int wbg_ws_replicas(const double* shifts, int nshift, const int* pts, int npt, const int* sup, int nsup,
                    const wbg_lattice* lat, double tol, int maxrep, int* count, int* repq, void* stream);
int wbg_r2k(const void* XF, int nfields, const int* pair_start, const int* r2, const int* slice_start,
            const int* pair_r1, const int* slice_r0, const void* ph0, const void* ph1, const void* ph2, int nblocks,
            int prec, void* workspace, size_t workspace_bytes, void* fields_out, const wbg_r2k_geom* g,
            void* stream);
/* wbg_r2k restricted to a list of elements: cols[c] = f*nw*nw + m*nw + n (0 <= c < ncols).
 * Only those elements of fields_out are written.  The mixed-precision path asks for the
 * lower triangle (m >= n) of the Hermitian fields and lets each consumer mirror the upper
 * triangle, so the fields are exactly Hermitian and the transform costs half.  H, AA and rotAA
 * are symmetrised as 1/2 (X + X^dagger) by the reference too (fourier/fft.py:183-186,
 * data_K/data_K_R.py:26,87); the derivatives of H are Hermitian analytically, so for them the
 * mirror removes only rounding noise. */
int wbg_r2k_columns(const void* XF, int nfields, const int* cols, int ncols, const int* pair_start, const int* r2,
                    const int* slice_start, const int* pair_r1, const int* slice_r0, const void* ph0, const void* ph1,
                    const void* ph2, int nblocks, int prec, void* workspace, size_t workspace_bytes, void* fields_out,
                    const wbg_r2k_geom* g, void* stream);

/* ---- stage 2: batched Hermitian eigensolver ---------------------------------------------
 * H: matrix k at H + k*strideH (complex128 elements), symmetrised as 1/2 (H + H^dagger).
 * mode 0: tridiagonalisation, eigenvalues and inverse iteration in FP64, back-transform in
 *         FP32, U complex64;
 * mode 1: everything in FP64, U complex128 (the plain FP64 path);
 * mode 2: tridiagonalisation, eigenvalues and inverse iteration in double-float arithmetic
 *         (pairs of FP32, 48-bit significand, on the FP32 pipe), back-transform in FP32,
 *         U complex64;
 * mode 3: as mode 2 with H given as double-float complex (wbg_r2k prec 2 output; the
 *         mixed-precision path).
 * mode | 4 (WBG_EIGH_LOWER): only the lower triangle (m >= n) of H is read and taken as the
 *         Hermitian matrix (imaginary part of the diagonal ignored) -- the output of
 *         wbg_r2k_columns on the lower triangle.
 * mode | 8 (WBG_EIGH_VALUES): eigenvalues only (np.linalg.eigvalsh; the tetrahedron corners,
 *         data_K/data_K_R.py:121-141); U is not written and may be NULL.
 * mode | 16 (WBG_EIGH_STAGE1): the tridiagonalisation only, kept in the workspace; a later call
 *         with mode | 32 (WBG_EIGH_STAGE2) and the same nw, nk, base mode and workspace finishes
 *         (eigenvalues, vectors; H is not read and may be NULL).  Lets a caller start
 *         independent work on another stream between the two stages.
 * mode | 64 (WBG_EIGH_PRECISE_VECTORS), modes 0, 2, 3: the Householder reflectors are kept and
 *         the back-transform runs in the solve's precision (FP64, double-float), U is rounded to
 *         complex64 once at the end -- eigenvectors as accurate as complex64 holds them, where the
 *         FP32 back-transform loses ~sqrt(nw) ulps.
 * mode | 64 | 128 (WBG_EIGH_DF64_VECTORS), modes 2, 3: as 64 with U kept in double-float complex
 *         (re.hi, re.lo, im.hi, im.lo floats per element, 16 bytes) for a double-float rotation.
 * mode | 256 (WBG_EIGH_REFINE), modes 2, 3 with nw <= 32, eigenvectors: the whole solve in FP32
 *         (H rounded to FP32), then one Ogita-Aishima refinement step against the double-float
 *         (mode 3) or FP64 (mode 2) H, with a Rayleigh-Ritz step inside clusters of close
 *         eigenvalues; U complex64.  Eigenvalues to ~1e-13 |H|, eigenvectors as accurate as
 *         complex64 holds them.  Not with 8, 64 or 128.  With the two-stage split, the STAGE2
 *         call reads H as well (the refinement), so H must still hold the matrices.
 * E [nk][nw] ascending (float64); U: matrix k at U + k*strideU, column n = eigenvector n.
 * errflag: device int, OR-ed with 1 when the QL iteration did not converge, and (WBG_EIGH_REFINE)
 *          with 4 when more than 8 eigenvalues of one matrix lay within 2^-8 max|lambda| of each
 *          other in a run (re-diagonalised 8 at a time: exact where the run is exactly degenerate,
 *          otherwise its eigenvalues keep the FP32 solve's accuracy), or when a matrix still needed
 *          a correction above 2^-12 in its second refinement step (a matrix needing one above 2^-12
 *          in the first step takes a second). */
#define WBG_EIGH_LOWER 4
#define WBG_EIGH_VALUES 8
#define WBG_EIGH_STAGE1 16
#define WBG_EIGH_STAGE2 32
#define WBG_EIGH_PRECISE_VECTORS 64
#define WBG_EIGH_DF64_VECTORS 128
#define WBG_EIGH_REFINE 256
int wbg_eigh_workspace_size(int nw, int nk, size_t* bytes);
int wbg_eigh_batched(const void* H, long long strideH, int nw, int nk, double* E, void* U, long long strideU,
                     int mode, void* workspace, size_t workspace_bytes, int* errflag, void* stream);

/* Allocation-free variant of wbg_eigh_batched (no counterpart in the reference).
 * For callers that cannot allocate device memory: a plugin inside a host application whose
 * memory manager owns the GPU's memory (a caching allocator, a fixed budget), a real-time loop
 * that forbids allocation after start-up (cudaMalloc / cudaFree may synchronise the device and
 * take unbounded time), or an FFI binding with no device allocator of its own.  The workspace
 * is a fixed file-scope device array of WBG_EIGH_NOALLOC_SCRATCH_BYTES that every GPU loading
 * the library keeps until process exit.  Same arguments, rules and results as
 * wbg_eigh_batched minus the workspace (U may be NULL with WBG_EIGH_VALUES), except that the
 * two-stage split WBG_EIGH_STAGE1 / WBG_EIGH_STAGE2 is refused (WBG_STATUS_BAD_ARGUMENT): any
 * other call between the stages would overwrite the shared array.  A batch needs
 *   nk * (16*nw*nw + 32*nw) + 1024 <= WBG_EIGH_NOALLOC_SCRATCH_BYTES
 * (nw = 32: nk <= 1920); larger batches return WBG_STATUS_TOO_LARGE without launching.
 * The first call on a device (and the first call after that device's context was destroyed
 * and recreated) looks up the array's device address with cudaGetSymbolAddress; make that
 * first call before any stream capture.  All calls share the array, which keeps the last
 * call's contents: calls whose work overlaps on the GPU race, so serialise them.  No device
 * memory is allocated or freed. */
#define WBG_EIGH_NOALLOC_SCRATCH_BYTES (32u << 20)
int wbg_eigh_batched_noalloc(const void* H, long long strideH, int nw, int nk, double* E, void* U,
                             long long strideU, int mode, int* errflag, void* stream);

/* ---- stage 3: U^dagger X U ----------------------------------------------------------------
 * X [nk][nFin][nw][nw] and U (matrix k at U + k*strideU) both complex128 (fp64 = 1), complex64
 * (fp64 = 0) or double-float complex (fp64 = 2: products in double-float, Xbar rounded to
 * complex64 -- the mixed path above nw = 32).
 * Xbar [nk][nFrot][nw][nw]: field f = U^dagger X[fsel[f]] U; herm[f] = 1: its Hermitian part;
 * herm[f] = 2: at least the diagonal of the Hermitian part (real) is written -- for fields
 * whose consumers read the diagonal only (rotA in Omega / Morb_Hpm).
 * herm[f] | 4: X[fsel[f]] holds only its lower triangle (wbg_r2k_columns output); it is read
 * as the Hermitian matrix with that lower triangle and a real diagonal.
 * fp64 == 0 and nw == 32 run on the tensor cores (tcgen05, products split into three TF32
 * terms, FP32 accumulation) when X is 16-byte aligned; other cases on the CUDA cores. */
int wbg_rotate(const void* U, long long strideU, const void* X, int nFin, const int* fsel, const int* herm,
               int nFrot, void* Xbar, int nw, int nk, int fp64, void* stream);

/* Device-side error word of the library (bitmask, sticky until cleared).
 * WBG_DEVICE_FLAG_TC_TIMEOUT: a tensor-core kernel's wait for its MMAs exceeded its 1 s bound;
 * that launch's results are invalid.  Synchronises the current device, then reads (and with
 * clear != 0 resets) the word. */
#define WBG_DEVICE_FLAG_TC_TIMEOUT 1
int wbg_device_flags(unsigned int* flags, int clear);

/* Failure detection of the tensor-core kernels (no counterpart in the reference).  Every mbarrier
 * wait of those kernels gives up after a bound (1 s by default), records
 * WBG_DEVICE_FLAG_TC_TIMEOUT, waits (at most 1 s) for the products it has issued, frees its
 * tensor memory and returns; the context stays usable.  wbg_tc_wait_limit sets the bound in ns
 * (for tests: a small bound makes waits run out); wbg_tc_wait_probe runs one such wait on an
 * mbarrier whose phase never completes and writes 0 to the device int *result when it ran out
 * (1 if it completed). */
int wbg_tc_wait_limit(unsigned long long ns);
int wbg_tc_wait_probe(int* result, void* stream);

/* ---- generic Fermi-level scan of additive group traces (calculators/static.py:60-169) ------
 * formula WBG_FORMULA_IDENTITY: group size (CumDOS / DOS, calculators/static.py:192-214), 1
 *   component; WBG_FORMULA_INVMASS: the inverse-mass tensor dV^b/dk_d (formula/elementary.py:28-34,
 *   Ohmic_FermiSea), Xbar: V at iV..iV+2, d^2H/dk_b dk_d at iW..iW+8, 9 components;
 *   WBG_FORMULA_VELVEL: in-group V^a V^b (formula/covariant.py:817-820, Ohmic_FermiSurf), 9;
 *   WBG_FORMULA_DIAG: Re X^c_nn of the 3-component field at iV (the spin expectation of
 *   calculators/static.py:217-228 Spin, formula/covariant.py:331-335), 3;
 *   WBG_FORMULA_VELVELVEL: in-group Re V^a V^b V^c (formula/covariant.py VelVelVel,
 *   NLDrude_Fermider2 of calculators/static.py:545-556), 27, (a, b, c) at 9 a + 3 b + c.
 * WBG_FORMULA_SPIN_OMEGA (the static spin Hall conductivity) goes through wbg_berry_shc (below).
 * sea != 0: Fermi-sea weights (fder 0), sea == 0: Fermi-surface groups only (fder >= 1; the
 * caller takes the finite differences over the extended levels).  hist [nEF][ncomp] (fixed point, see
 * "Histograms" below)
 * is accumulated; component (b, d) at 3 b + d.  Xbar may be NULL for WBG_FORMULA_IDENTITY. */
#define WBG_FORMULA_IDENTITY 0
#define WBG_FORMULA_INVMASS 1
#define WBG_FORMULA_VELVEL 2
#define WBG_FORMULA_DIAG 6
#define WBG_FORMULA_VELVELVEL 7
#define WBG_FORMULA_SPIN_OMEGA 8
int wbg_berry_scan(const double* E, const void* Xbar, int nFbar, int iV, int iW, int nw, int nk, const wbg_scan* scan,
                   int formula, int sea, void* hist, int fp64, void* stream);

/* ---- in-group matrix products (formula/formula.py:121-151 FormulaProduct) -----------------
 * Replaces the StaticCalculator trace (calculators/static.py:60-169) of the product formulas of
 * formula/covariant.py:798-865: VelOmega (BerryDipole_FermiSurf / NLAHC_FermiSurf,
 * calculators/static.py:449-469), MassVel (NLDrude_FermiSurf, :532-542), VelMassVel / MassMass
 * (Hall_classic_FermiSurf / FermiSea, :407-446), VelSpin (GME_spin_FermiSurf, :340-350), VelHplus
 * (GME_orb_FermiSurf, :266-281), OmegaS (AHC_Zeeman_spin, :605-615), OmegaOmega (:618-623),
 * OmegaHplus (AHC_Zeeman_orb, :626-644), and of the single factor DerSpin (GME_spin_FermiSea,
 * :322-337).  factor[0..nfactors) lists the factors in product order: WBG_FACTOR_VEL (V^a, 3
 * components), WBG_FACTOR_SPIN (S^a, 3), WBG_FACTOR_OMEGA (the nn block of Omega^c,
 * formula/covariant.py:161-203, 3), WBG_FACTOR_MASS (the nn block of the inverse mass M^{bd},
 * formula/elementary.py:28-34, 9 at 3 b + d), WBG_FACTOR_DERSPIN (the generalised derivative of
 * S, (a, d) at 3 a + d, formula/covariant.py:338-342) and WBG_FACTOR_HPLUS (Morb_Hpm with sign +1,
 * formula/covariant.py:375-449, 3); internal_terms / external_terms select the terms of Omega and
 * Morb_Hpm.  Per group G the trace Re sum_{n[, p[, q]] in G} F1_n(p) [F2_p(q) [F3_qn]] is binned as
 * wbg_berry_scan (sea != 0: the Fermi-sea group), components of the factors one after another
 * ((i d2 + j) d3 + m), at most 81.  Field indices into Xbar (full matrices, not lower triangles;
 * -1 when unused): V (3); A (3) and O = rotA (3) for Omega or Morb_Hpm with external terms, and B,
 * C (3 each) for Morb_Hpm; W = d^2H/dk_b dk_d (9) for a mass factor; S (3) for a spin factor and S
 * with dS = dS^a/dk_d (9, 3 a + d) for DerSpin.  wbg_product_values writes the per-band values of
 * the tetrahedron method instead (as wbg_band_values). */
#define WBG_FACTOR_VEL 0
#define WBG_FACTOR_SPIN 1
#define WBG_FACTOR_OMEGA 2
#define WBG_FACTOR_MASS 3
#define WBG_FACTOR_DERSPIN 4
#define WBG_FACTOR_HPLUS 5
typedef struct {
  int nfactors;   /* 1 to 3 */
  int factor[3];  /* WBG_FACTOR_* in product order */
  int internal_terms, external_terms;
  int V, A, O, W, S, B, C, dS;
} wbg_product_spec;
int wbg_berry_product(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                      const wbg_scan* scan, int sea, void* hist, int fp64, void* stream);
int wbg_product_values(const double* E, const void* Xbar, int nFbar, const wbg_product_spec* spec, int nw, int nk,
                       double degen_thresh, const signed char* sel, double* P, int fp64, void* stream);

/* ---- tetrahedron method (calculators/static.py:80-125 with tetra=True; grid/tetrahedron.py:
 * 15-281 TetraWeightsParal; corner energies data_K/data_K_R.py:121-141) ---------------------
 * The parallelepiped k +- delta/2 (delta = 1/(NKdiv NKFFT) per axis) around each k-point is cut
 * into 12 tetrahedra.  Its 8 corners are points of the dense grid shifted by +delta/2: corner
 * block c (c = 0..NKdiv-1 per axis, flat index (c0 div1 + c1) div2 + c2) is the FFT grid at
 * shift (c + 1/2) delta.  The caller computes their eigenvalues once (wbg_eigh_batched with
 * WBG_EIGH_VALUES) into Ecorner[row][k][n] and passes corner_slot[flat corner block] = row for
 * every corner block the batch touches (blocks i and i-1 per axis, i-1 = NKdiv-1 at i = 0).
 * blocks[b]: flat division-grid index (C order) of batch block b; E [nblocks*nk][nw] the
 * k-point energies of the batch (blocks in that order, k in C order of the FFT grid). */
typedef struct {
  int div[3];    /* NKdiv */
  int fft[3];    /* NKFFT */
  int per_block; /* != 0: every block has its own 8 corner grids (refined blocks, whose cell
                    differs from the grid's): corner s of k-point kl of block b at
                    Ecorner row corner_slot[blocks[b]] * 8 + s, index kl */
} wbg_tetra_grid;

/* Bands that take part (tetrahedron.py:215-262 weights_all_band_groups, Emin = -inf):
 * sel [nblocks*nk][nw] = 1 when the band's degenerate group (by E, gap > degen_thresh) is in
 * the window (largest corner energy >= EF0, smallest <= EF1); with sea != 0 (Fermi-sea
 * calculators) = 2 for bands [0, bandmax), bandmax = 1 + the last band whose corners all lie
 * below EF0, capped at the first in-range group; else 0. */
int wbg_tetra_select(const double* E, const double* Ecorner, const int* corner_slot, const int* blocks, int nblocks,
                     const wbg_tetra_grid* grid, int nw, double EF0, double EF1, double degen_thresh, int sea,
                     signed char* sel, void* stream);

/* Per-band formula values for the tetrahedron method: the group traces of the histogram
 * kernels, written per band instead of binned.  P [nk][nw][ncomp] = trace of the band's group
 * / group size for sel 1, the trace of the sea group [0, bandmax) on band 0 for sel 2 (Morb:
 * T(bandmax) - T(0)), 0 otherwise.  formula: WBG_FORMULA_IDENTITY / INVMASS / VELVEL / DIAG
 * (as wbg_berry_scan; DIAG reads the field at fields->V), WBG_FORMULA_OMEGA (wbg_berry_omega, 3), WBG_FORMULA_DEROMEGA
 * (wbg_berry_deromega, 9, (c, d) at 3 c + d), WBG_FORMULA_MORB (wbg_berry_morb, 3).  fields:
 * field indices into Xbar (unused entries ignored); fp64 0 / 1 as the histogram kernels. */
#define WBG_FORMULA_OMEGA 3
#define WBG_FORMULA_DEROMEGA 4
#define WBG_FORMULA_MORB 5
typedef struct {
  int V, A, O, W, dA, dO, B, C;
} wbg_field_index;
int wbg_band_values(const double* E, const void* Xbar, int nFbar, const wbg_field_index* fields, int nw, int nk,
                    int formula, int internal_terms, int external_terms, double degen_thresh,
                    const signed char* sel, double* P, int fp64, void* stream);

/* Weighted sum over the bands of every k-point (ncomp = 1..81 components per band):
 * sum_n P[k][n][c] w_n(E_F) with the band weight w_n = 1/12 sum over the 12 tetrahedra
 * (k-point + 3 corners) of the linear-tetrahedron occupation (der 0) or its E_F derivative
 * (der 1) at efermi[0..nEF) -- weight 1 for sel 2 bands (der 0).  hist [nEF][ncomp] is
 * accumulated in difference form (hist[i] += P (w(i) - w(i-1))): wbg_scan_finalize turns it
 * into the sum.  ascending != 0: efermi is sorted ascending and only the levels between a
 * band's smallest and largest corner energy are evaluated.  fp64 = 1: the reference's FP64
 * arithmetic (der 1 from its expanded cubic); fp64 = 0 (mixed precision): energies relative
 * to each band's lowest one as double-float pairs, then FP32 relative to each tetrahedron's
 * lowest corner (~1e-7 relative error per weight; der 1 from the product rule on the
 * piecewise form, free of the cubic's cancellation). */
int wbg_tetra_accumulate(const double* E, const double* Ecorner, const int* corner_slot, const int* blocks,
                         int nblocks, const wbg_tetra_grid* grid, int nw, const signed char* sel, const double* P,
                         int ncomp, const double* efermi, int nEF, int der, int ascending, int fp64, void* hist,
                         void* stream);

/* ---- tabulation (calculators/tabulate.py:21-52 Tabulator with Energy, Velocity,
 * BerryCurvature; evaluate_k.py:9-16 "energy", "band_gradients", "berry_curvature") ----------
 * For every k and band n, the average over n's degenerate group (gap > degen_thresh) of
 * E, Re V^a_nn and the Omega trace: tab [nk][nw][7] = (E, V_x, V_y, V_z, Omega_x, Omega_y,
 * Omega_z) (double).  Xbar and fp64 as wbg_berry_omega (fp64 0 or 1). */
int wbg_berry_tabulate(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                       double degen_thresh, int internal_terms, int external_terms, double* tab, int fp64,
                       void* stream);

/* ---- Histograms (every formula kernel, the tetrahedron accumulation, wbg_kubo / wbg_dynamic) ----
 * A histogram of n entries is 2 n + 1 64-bit words, zeroed by the caller and accumulated (never
 * cleared) by the kernels: entry i is the 128-bit two's-complement integer sum of floor(v 2^60)
 * over its contributions v, low word at [2 i], high word at [2 i + 1]; word [2 n] counts
 * contributions that were not finite (the readers then return NaN throughout).  Integer sums
 * commute, so a histogram holds the same bits whatever the order of the atomic adds -- over
 * threads, blocks, launches and concurrent requests.  Resolution 2^-60 absolute, range 2^67.
 * Value of an entry: hi 2^4 + ((lo >> 32) 2^-28 + (lo mod 2^32) 2^-60) (wbg_scan_finalize). */

/* ---- stage 4: Berry curvature traces + Fermi-level histogram ----------------------------
 * Xbar [nk][nFbar][nw][nw]: velocity dH/dk at iV..iV+2, A at iA..iA+2, rotA at iO..iO+2.
 * hist [scan.nEF][3] (fixed point, see "Histograms") is accumulated.
 * fp64: 1 complex128 Xbar; 0 complex64; 2 complex64 whose V and A are exactly Hermitian
 * (the mixed path's rotation output) -- then the (l, n) elements are taken as conj(X_nl) and
 * every load is a coalesced row segment (nw <= 32). */
int wbg_berry_omega(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int nw, int nk,
                    const wbg_scan* scan, int internal_terms, int external_terms, void* hist, int fp64,
                    void* stream);

/* Orbital moment, Morb_Hpm = Morb_H + E_av Omega (formula/covariant.py:375-449), the non-additive
 * formula of the Morb calculator (calculators/static.py:231-247): group values are differences
 * of traces over [0, n) at the group borders (calculators/static.py:109-117).  Xbar holds
 * V at iV, A (Hermitian part) at iA, rotA at iO, B at iB, C at iC (3 fields each).
 * hist [scan.nEF][3] is accumulated.  The Morb calculator combines it with a wbg_berry_omega
 * histogram: M(E_F) = [cumsum(hist_Hpm) - 2 E_F cumsum(hist_Omega)] * factor / nk. */
int wbg_berry_morb(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iB, int iC, int nw,
                   int nk, const wbg_scan* scan, int internal_terms, int external_terms, void* hist, int fp64,
                   void* stream);

/* Berry-curvature dipole, DerOmega (formula/covariant.py:212-259) with DerDcov
 * (formula/elementary.py:55-70) and the generalised derivatives of A and rotA
 * (formula/formula.py:95-118); BerryDipole_FermiSea (calculators/static.py:472-487).
 * Xbar: V at iV (3), A at iA (3), rotA at iO (3), d_a d_b H at iW (9, [a][b]),
 * d_d A_b at idA (9, [b][d]), d_d rotA_c at idO (9, [c][d]).
 * hist [scan.nEF][3][3] ([c][d], before the calculator's swap of the last two axes).
 * fp64: 1 complex128 Xbar and FP64 arithmetic; 0 complex64 Xbar, FP32 arithmetic; 2 complex64
 * Xbar, double-float arithmetic (the mixed path). */
int wbg_berry_deromega(const double* E, const void* Xbar, int nFbar, int iV, int iA, int iO, int iW, int idA,
                       int idO, int nw, int nk, const wbg_scan* scan, int internal_terms, int external_terms,
                       void* hist, int fp64, void* stream);

/* Kubo optical conductivity (calculators/dynamic.py:71-114,170-196).
 * Groups over all bands (degen_thresh); for every ordered pair of groups not pruned by
 * `nonzero`, f_w(E1,E2) f_E(E1,E2) M^{ab} is added to out[iEF][iw][a][b] (complex: real and
 * imaginary part each a fixed-point entry of "Histograms", 2 * nEF*nOmega*9 entries; accumulated,
 * not normalised: the calculator multiplies by factor_opt / (nk * V)).
 * efermi [nEF] and omega [nOmega] are device arrays; gaussian != 0 selects the Gaussian
 * smearing of the imaginary part, else Lorentzian.  Xbar: V at iV, A at iA (3 fields each). */
typedef struct {
  double EFmin, EFmax, kBT, eta, degen_thresh;
  int nEF, nOmega, gaussian, reserved;
} wbg_kubo_params;
int wbg_kubo_workspace_size(int nw, int nk, int nEF, size_t* bytes);
int wbg_kubo(const double* E, const void* Xbar, int nFbar, int iV, int iA, int nw, int nk, int external_terms,
             const wbg_kubo_params* params, const double* efermi, const double* omega, void* workspace,
             size_t workspace_bytes, void* out, int fp64, void* stream);

/* ---- dynamic calculators (calculators/dynamic.py:26-360) -------------------------------------
 * The Kubo pair scan of wbg_kubo for every formula of DynamicCalculator: per k-point, groups
 * over all bands (degen_thresh), each ordered pair (G1, G2) kept by `nonzero` (dynamic.py:65-69;
 * JDOS: E1 < EFmax, E2 > EFmin, omega_min - 5 eta < E1 - E2 < omega_max + 5 eta, :158-162) adds
 * f_w(E1, E2) (FD(E2) - FD(E1)) M^c to out[iEF][iw][c] (complex, as wbg_kubo's: fixed-point real and
 * imaginary parts, accumulated, unnormalised).
 * formula / M^c (n in G1, m in G2 summed; A = i D + Abar with Abar only when external_terms):
 *   WBG_DYN_OPTCOND    i A^a_nm A^b_mn, c = 3 a + b (OpticalConductivity, :170-196; = wbg_kubo)
 *   WBG_DYN_JDOS       1, one component (JDOS, :133-162)
 *   WBG_DYN_SHC_*      Im(J^{as}_nm (-i A^b_mn)), c = 9 a + 3 b + s, J the spin current
 *                      (J' + J'^dagger) / 2 of formula/covariant.py:721-756 of kind SIMPLE / QIAO /
 *                      RYOO (QIAO and RYOO need external_terms); f_w = 1 / (E1 - E2 - w - i eta) / 2
 *                      (SHC, :199-236)
 *   WBG_DYN_SHIFT      -Im(dA^{ca}_nm A^b_mn) + (b <-> c), c-index 9 a + 3 b + c, dA the generalised
 *                      derivative with the principal-value D of broadening sc_eta (ShiftCurrent,
 *                      :239-316); f_w = smear(E1 - E2 - w) + smear(E2 - E1 - w), real
 *   WBG_DYN_INJECTION  (v^a_n - v^a_m) A^b_nm A^c_mn, 9 a + 3 b + c (InjectionCurrent, :319-360);
 *                      f_w = smear(E1 - E2 - w)
 * smear: Lorentzian or (params->gaussian) Gaussian of width params->eta (utility.py:147-168).
 * spec: the first Xbar field of each quantity (-1 where unused): V (3), A (3), W = d2H (9),
 * dA = dAbar/dk (9, (c, d) at 3 c + d), S = SS (3), SH (3), SA, SHA, SR, SHR (9, (a, s) at
 * 3 a + s).  Xbar may be NULL for JDOS.  ncomp: wbg_dynamic_ncomp(formula) (9, 1 or 27). */
#define WBG_DYN_OPTCOND 0
#define WBG_DYN_JDOS 1
#define WBG_DYN_SHC_SIMPLE 2
#define WBG_DYN_SHC_QIAO 3
#define WBG_DYN_SHC_RYOO 4
#define WBG_DYN_SHIFT 5
#define WBG_DYN_INJECTION 6
typedef struct {
  int formula, external_terms;
  int V, A, W, dA, S, SH, SA, SHA, SR, SHR;
  double sc_eta;               /* ShiftCurrent */
  double omega_min, omega_max; /* JDOS `nonzero` window */
} wbg_dynamic_spec;
int wbg_dynamic_ncomp(int formula);
int wbg_dynamic_workspace_size(int formula, int nw, int nk, int nEF, size_t* bytes);
int wbg_dynamic(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* spec, int nw, int nk,
                const wbg_kubo_params* params, const double* efermi, const double* omega, void* workspace,
                size_t workspace_bytes, void* out, int fp64, void* stream);

/* Static spin Hall conductivity (calculators/static.py:647-660, formula SpinOmega of
 * formula/covariant.py:759-788): the Fermi-sea scan (as wbg_berry_scan with sea != 0) of the
 * additive group traces  sum_{n in G} sum_{l not in G} -2 Im( J^{as}_nl / (E_n - E_l)
 * (D^b_ln - i Abar^b_ln) ), component 9 a + 3 b + s, J the spin current of kind
 * spin->formula (WBG_DYN_SHC_SIMPLE / QIAO / RYOO) from the fields named in spin (see
 * wbg_dynamic_spec; Abar only with spin->external_terms).  hist [nEF][27] accumulated. */
int wbg_berry_shc(const double* E, const void* Xbar, int nFbar, const wbg_dynamic_spec* spin, int nw, int nk,
                  const wbg_scan* scan, void* hist, int fp64, void* stream);

/* cumulative sum over levels times scale: out[i][c] = scale * sum_{j<=i} hist[j][c] (double),
 * hist in the fixed-point layout of "Histograms"; NaN throughout when it counted a non-finite
 * contribution */
int wbg_scan_finalize(const void* hist, int nEF, int ncomp, double scale, double* out, void* stream);

/* ---- launch-shape table of the autotuner (no reference counterpart: the reference's numpy
 * calls have no launch shapes) ------------------------------------------------------------------
 * A host-side table, per (parameter, variant, nw), of launch shapes that a tuner measured to be
 * fastest; 0 (the initial value) selects the built-in occupancy heuristic.  Parameters:
 *   WBG_TUNE_EIGH_TRIDIAG_GROUP  matrices per block of the tridiagonalisation   variant: eigh mode & 3,
 *                                4 for modes 2 / 3 with WBG_EIGH_PRECISE_VECTORS,
 *                                5 for modes 2 / 3 with WBG_EIGH_REFINE
 *   WBG_TUNE_EIGH_QL_BLOCK       matrices (threads) per block of the QL sweep   variant: eigh mode & 3
 *   WBG_TUNE_EIGH_VECTORS_GROUP  matrices per block of the inverse iteration and
 *                                back-transform                                variant: eigh mode & 3
 *   WBG_TUNE_ROTATE_KPOINTS      k-points per block of the CUDA-core tiled U^dagger X U  variant: fp64
 *   WBG_TUNE_ROTATE_ENGINE       1 tensor cores, warp-specialised (two tiles in flight), 2 CUDA
 *                                cores, 3 tensor cores one tile at a time (the built-in choice;
 *                                where they serve the case)                    variant: fp64
 *   WBG_TUNE_KUBO_ENGINE         the mixed path's 9- and 27-component Kubo band sums: 1 tensor
 *                                cores (the built-in choice), 2 CUDA-core register-tiled GEMM
 *                                                                               variant 0, nw 1
 * wbg_tune_candidates lists the values that fit the launch limits of (parameter, nw, variant);
 * wbg_tune_set accepts 0 or one of them (else WBG_STATUS_BAD_ARGUMENT), so every launch shape
 * the table can select is one the kernels accept.  Results do not depend on the eigensolver and
 * tiled-rotation shapes (each matrix or k-point is computed by the same code whatever the
 * grouping); the rotation engine changes the FP32 rounding (both within the FP32 path's error
 * budget).  The table is process-wide: set it before launching work that should use it. */
#define WBG_TUNE_EIGH_TRIDIAG_GROUP 0
#define WBG_TUNE_EIGH_QL_BLOCK 1
#define WBG_TUNE_EIGH_VECTORS_GROUP 2
#define WBG_TUNE_ROTATE_KPOINTS 3
#define WBG_TUNE_ROTATE_ENGINE 4
#define WBG_TUNE_KUBO_ENGINE 5
#define WBG_TUNE_NPARAM 6
int wbg_tune_candidates(int param, int nw, int variant, int* values, int capacity, int* count);
int wbg_tune_set(int param, int nw, int variant, int value);
int wbg_tune_get(int param, int nw, int variant, int* value);

/* ---- measurement helper (no reference counterpart) ----------------------------------------
 * FMA throughput probe giving the roofline denominator of FP64- / FP32-pipe-bound kernels:
 * blocks*threads threads run 8 independent FMA chains of `iters` steps; out holds
 * blocks*threads elements of the probed type; *flops_per_launch receives the flop count. */
int wbg_probe_fma(int fp64, int blocks, int threads, int iters, void* out, double* flops_per_launch, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* WBGPU_H */
