/*
 * scalit_gb300 -- GB300 (sm_103a) implementation of ScalIT's iterate hot path:
 * the H*X product on a direct-product DVR grid, the OSB block-Jacobi
 * preconditioner P*X, QMR inner solves and the PIST eigensolver.
 *
 * C ABI.  Plain pointers and sizes only.  Arrays are column-major with the
 * reference's level order (level 1 varies fastest).  Unless a function name
 * ends in _device, array arguments are HOST memory owned by the caller; the
 * library copies them.  The _device variants take device pointers on the
 * context's device and run on the context's stream.
 *
 * Status convention: functions returning int return 0 (or a positive count)
 * on success and a negative SCALIT_E* code on failure, with a message
 * available from scalit_last_error().  Solver entry points keep the
 * reference's sign conventions (QMR: +iterations converged, -iterations not
 * converged, -1..-4 breakdown; PIST: +Krylov size converged, -size not
 * converged, 0 bad parameters).
 */
#ifndef SCALIT_GB300_H
#define SCALIT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SCALIT_FMAX 20

/* error codes */
#define SCALIT_OK 0
#define SCALIT_EINVAL (-101)     /* bad argument */
#define SCALIT_ECUDA (-102)      /* CUDA runtime / library failure */
#define SCALIT_ENOMEM (-103)     /* device allocation failed */
#define SCALIT_ESTATE (-104)     /* call out of order (e.g. P*X before the build) */
#define SCALIT_EUNSUP (-105)     /* option not supported */
#define SCALIT_ENONFINITE (-106) /* NaN/Inf found in an input */

/* operator kinds (sHC / sPC; src/iterate/module/osb.data.h TA0, TA1) */
#define SCALIT_TA0 0 /* H*X (no shift)        */
#define SCALIT_TA1 1 /* (H - E0)*X            */
/* nType codes of the complex forms with absorbing potentials
 * (src/iterate/module/osb.data.h:18-22) */
#define SCALIT_TAAP0 2   /* (H + i AP) X          */
#define SCALIT_TMAP0 3   /* (H - i AP) X          */
#define SCALIT_TAAP 100  /* (H - E0 + i AP) X     */
#define SCALIT_TAAPP 101 /* (H - E0 + i APP) X    */
#define SCALIT_TAAPR 102 /* (H - E0 + i APR) X    */
#define SCALIT_TMAP 200  /* (H - E0 - i AP) X     */
#define SCALIT_TMAPP 201 /* (H - E0 - i APP) X    */
#define SCALIT_TMAPR 202 /* (H - E0 - i APR) X    */

/* preconditioner kernels (sOSB; osb.data.h TOSB..TOSBD2) */
#define SCALIT_TOSB 1   /* 1/(EIG0 - E0)                           */
#define SCALIT_TOSBD1 2 /* +-1/DE inside the window |EIG0-E0| <= DE */
#define SCALIT_TOSBD2 3 /* 1/(+-alpha + beta (EIG0-E0)) in window   */
#define SCALIT_TOSBW 4  /* exact (H - E0)^-1 on a window of states    */

/* engine of the FP64 H*X level products */
#define SCALIT_FP64_DFMA 0   /* FP64 pipe (strided GEMM on CUDA cores)                 */
#define SCALIT_FP64_TENSOR 1 /* 7-bit digit slices on the BF16 tensor cores (tcgen05), */
                             /* exact FP32 group sums, FP64 recombination (default)     */

/* engine of the FP32 (inner-solve) level products and preconditioner rotations */
#define SCALIT_FP32_SIMT 0   /* FP32 CUDA cores (strided GEMM)                         */
#define SCALIT_FP32_TENSOR 1 /* split-BF16 x3 on the tensor cores (tcgen05), FP32 sums */
#define SCALIT_FP32_TENSOR_PX 2 /* preconditioner rotations on the tensor cores, H*X on
                                   the CUDA cores: the operator keeps FP32 accuracy (the
                                   QMR's attainable residual), the preconditioner, whose
                                   accuracy only sets the convergence rate, takes the
                                   faster engine                                         */
#define SCALIT_FP32_TENSOR16 3 /* H*X levels in split-FP16 x3 on the tensor cores with
                                  exponent scaling (per vector and per matrix column;
                                  ~22 significant bits, the accuracy of the CUDA-core
                                  GEMM), persistent pipelined kernels; preconditioner
                                  rotations in split-BF16 x3                          */

/* arithmetic of the QMR inner solves */
#define SCALIT_PREC_FP64 0
#define SCALIT_PREC_FP32 1
/* FP32 QMR solves under FP64 iterative refinement: x += QMR32(b - (H - E0) x)
 * with the residual formed by an FP64 H*X, until the FP64 residual meets the
 * tolerance (QMR solves only, not the shifted batches) */
#define SCALIT_PREC_FP32_REFINED 2

typedef struct scalit_ctx scalit_ctx;

/* ---------------------------------------------------------------- context --
 * Replaces the module state set up by initOSB/calOSB + loadInitData
 * (src/iterate/module/osb.f90:17-20, osb.init.h:2-49, osb.io.h:2-42) and the
 * MPI counterparts initMOSB/loadInitData (mosb3.init.h:5-20, posb.io.h:6-70).
 * nlevel = sF, sizes = sN(1:sF), dep = sDEP(1:sF) (dep[0] is forced false as
 * in osb.print.h:198-199), ndvr = sNDVR.  device = CUDA ordinal.
 */
int scalit_create(scalit_ctx **ctx, int nlevel, const int *sizes, const int *dep, int ndvr,
                  int device);
void scalit_destroy(scalit_ctx *ctx);
const char *scalit_last_error(void);
long long scalit_npoints(const scalit_ctx *ctx);  /* myLen */
long long scalit_h0_len(const scalit_ctx *ctx);   /* myH0%mLen */
long long scalit_dep_len(const scalit_ctx *ctx);  /* myDEP%mLen */
long long scalit_vosb_len(const scalit_ctx *ctx); /* myVOSB%mLen */

/* Upload H0 (concatenated level matrices), RES (diagonal potential), DEP
 * (concatenated dependent-level factors; may be NULL if no level depends)
 * and OUTH (outermost per-point matrices when ndvr; else NULL).  EIG0 is
 * initialised to RES (loadRESEig, osb.io.h:71-77).  Non-finite input values
 * are rejected with SCALIT_ENONFINITE. */
int scalit_load(scalit_ctx *ctx, const double *H0, const double *RES, const double *DEP,
                const double *OUTH);
/* The CUDA stream (cudaStream_t) all of the context's work is queued on.
 * scalit_set_stream replaces it with a caller-owned stream (NULL restores
 * the context's own); the _device entry points are then ordered on it. */
void *scalit_get_stream(const scalit_ctx *ctx);
int scalit_set_stream(scalit_ctx *ctx, void *stream);
/* Engine of the FP64 H*X level products (SCALIT_FP64_DFMA or SCALIT_FP64_TENSOR).
 * Levels with more than 256 points, and the per-point outer layer, always use
 * the FP64 pipe. */
int scalit_set_fp64_mode(scalit_ctx *ctx, int mode);
/* Engine of the FP32 level products and preconditioner rotations
 * (SCALIT_FP32_SIMT, SCALIT_FP32_TENSOR, SCALIT_FP32_TENSOR_PX or
 * SCALIT_FP32_TENSOR16; levels above 256 points stay on the CUDA cores, and
 * SCALIT_FP32_TENSOR16 levels whose matrix does not fit one persistent tile
 * too).  Split-BF16 x3 carries ~16 significant bits (H*X relative error ~4e-6
 * against ~2e-7 on the CUDA cores); split-FP16 x3 with exponent scaling
 * carries ~22.  No reference counterpart: the reference has no FP32 path. */
int scalit_set_fp32_mode(scalit_ctx *ctx, int mode);
/* Precision of the Jacobi sweeps of the next scalit_build_osb calls:
 * SCALIT_PREC_FP64 (default, the reference's HosbDiag/MJACOBI) or
 * SCALIT_PREC_FP32 for a preconditioner that only feeds FP32 inner solves.
 * With FP32, the levels whose blocks hold one matrix each (the grid's first
 * level, where the build spends most of its time) sweep with angles,
 * rotations and V in FP32, and the outer levels' stacked matrices are
 * rotated in FP32 with their angles and V in FP64; EIG0 and the sweep test
 * are FP64 throughout.  No reference counterpart. */
int scalit_set_build_precision(scalit_ctx *ctx, int precision);
/* Storage of the first level's preconditioner matrices for the FP32 P*X:
 * bits = 32 (default, FP32) or 16 (an FP16 copy, made now and after every
 * scalit_build_osb / scalit_set_osb; first levels of a multiple of 8
 * points).  The FP32 P*X streams those matrices once per application -- the
 * largest array of the solve -- so FP16 halves its traffic; the rounding of
 * the eigenvectors (~2^-11) perturbs the preconditioner, not the operator,
 * so FP32 inner solves under FP64 refinement converge to the same result.
 * The FP64 P*X and the batched (several shifts) P*X keep FP32/FP64.  No
 * reference counterpart. */
int scalit_set_fp32_px_storage(scalit_ctx *ctx, int bits);
/* sOSBW%mE0: the shift of (H - E0) and of the preconditioner. */
int scalit_set_shift(scalit_ctx *ctx, double e0);
/* sOSB kernel kind with sOSBW%mDE and sOSBW%mBeta.  SCALIT_TOSBW needs a
 * window made by scalit_build_osbw / scalit_set_osbw for the current
 * preconditioner (SCALIT_ESTATE otherwise). */
int scalit_set_precond(scalit_ctx *ctx, int osb_kind, double de, double beta);

/* ---------------------------------------------------------------- H * X ---
 * MYHX (src/iterate/module/osb.hx.h:71-110; MPI mosb3.hx.h:6-66):
 *   Y = (RES - E0 [ntype==TA1]) .* X + sum_level H_level X
 * for nvec vectors stored one after another (each npoints long).
 * X and Y must not overlap. */
int scalit_hx(scalit_ctx *ctx, int ntype, int nvec, const double *X, double *Y);
int scalit_hx_device(scalit_ctx *ctx, int ntype, int nvec, const double *dX, double *dY);
/* Measurement aid, no counterpart in the reference: reps applications of
 * scalit_hx_device (precision SCALIT_PREC_FP64, on double vectors) or
 * scalit_hx_f32_device (SCALIT_PREC_FP32, float vectors) to nvec <= 64
 * vectors, with a CUDA event on the context's stream before every level's
 * launch; ms[level - 1] receives each level's average duration in ms. */
int scalit_hx_level_times(scalit_ctx *ctx, int precision, int ntype, int nvec, const void *dX, void *dY,
                          int reps, float *ms);
/* One level of MYHX on device vectors: Y (+)= H_level X (level is 1-based;
 * a dependent level is scaled by its DEP factors, H1X_DEP / H2X, hpx.f90:21-35;
 * otherwise H1X_XYZ, hpx.f90:5-18).  accumulate != 0 adds into Y. */
int scalit_level_device(scalit_ctx *ctx, int level, int accumulate, const double *dX, double *dY);
/* The same operator in FP32 (the QMR inner-solve arithmetic). */
int scalit_hx_f32_device(scalit_ctx *ctx, int ntype, int nvec, const float *dX, float *dY);

/* ------------------------------------------------- OSB preconditioner -----
 * myDiag (src/iterate/module/osb.diag.h:53-151; MPI posb.diag.h:53-198):
 * for level = sF..1 initialise HOSB (HOSBINIT_DEP/XYZ, hinitdep.f90:10-34,
 * hinitxyz.f90:7-29), run the joint block-Jacobi sweeps of HosbDiag
 * (hosbdiag.f90:5-75, jacobi.f90:2-83, vupdate.f90:4-36) until
 * |d offdiag| <= bjtol * offdiag_0 or bjmax sweeps, and take EIG0 from the
 * rotated diagonal.  stats (may be NULL) receives 5 numbers per level: min
 * and max Jacobi efficiency, their sum, the sum of squared diagonals and the
 * sum of sweep counters (the reference's eff(1:5)). */
int scalit_build_osb(scalit_ctx *ctx, int bjmax, double bjtol, double *stats);
/* The CUDA-core GEMM tile the load-time autotuner picked for each level:
 * picks[(prec * sF + level) * 2 + many], prec 0 = FP64 / 1 = FP32, many 0 = one
 * vector / 1 = a block of 16; 0 = 128x128 (FP32) / 64x64 (FP64) tiles,
 * 1 = the half-size tiles, -1 = not tuned (that engine is not used there).
 * No reference counterpart (the reference has one loop order). */
int scalit_tile_picks(scalit_ctx *ctx, int *picks);
/* Wall seconds spent on each level (sF entries, level 1 first) by the last
 * scalit_build_osb; the reference prints the whole build's time only
 * (osb.progDiag.h:40-47). */
int scalit_build_times(scalit_ctx *ctx, double *seconds);
/* Self-test of the kernels' bounded waits: a one-CTA kernel waits `seconds`
 * (0 < seconds <= 10) on an mbarrier that nothing completes, records the
 * expiry in the context's error flag and returns; the call reports it as the
 * product kernels' expiry is reported (SCALIT_ECUDA with a message) and the
 * context stays usable.  No reference counterpart. */
int scalit_selftest_wait(scalit_ctx *ctx, double seconds);
/* Copy the preconditioner out (VOSB: scalit_vosb_len doubles, EIG0: npoints)
 * or in (sVOSB < 0 path: loadVOSB/loadEig, osb.io.h:124-208). */
int scalit_get_osb(scalit_ctx *ctx, double *VOSB, double *EIG0);
int scalit_set_osb(scalit_ctx *ctx, const double *VOSB, const double *EIG0);

/* OSBW window preconditioner, bound-state job: initOSBW
 * (src/iterate/module/osb.osbw.h:2-50) after the preconditioner build.
 * The window width is adjusted (adjustWinSize, osb.osbw.h:118-145) until
 * exactly `count` states satisfy |EIG0 - e0| <= de; *de is the starting width
 * on entry and the final width on return.  HW(i, j) = <V_i | H | V_j> over the
 * window's basis vectors with H = MYHX(TA0) and EIG0 on the diagonal
 * (getVOSBH0, osb.hij.h:128-159); HWR = HW - shift I, shift = e0 for
 * npc == SCALIT_TA1 and 0 for SCALIT_TA0, is inverted once (createWH,
 * osb.pij.h:6-45, factors it for DSYTRS; here its symmetric eigen-decomposition
 * gives HWR^-1, equal to the factor's solve to rounding) and the TOSBW kernel
 * is selected for P*X (osb.px.h:191-206).
 * *hwlen (may be null) receives the window size.  Errors: SCALIT_ESTATE
 * before the preconditioner exists; SCALIT_EINVAL for count outside 1..N,
 * de <= 0, no width holding exactly count states within 2000 steps (tied
 * EIG0 values: the reference loops forever there) or a singular HWR (an
 * exactly zero eigenvalue, where DSYTRF reports info > 0 and createWH fails);
 * SCALIT_ENOMEM when the count basis vectors
 * (count x npoints doubles) do not fit.  Building the preconditioner again,
 * set_osb or load leaves the window stale: P*X with TOSBW then returns
 * SCALIT_ESTATE until the window is made again.  scalit_set_shift does not
 * refactor HWR (the reference factors it once, at initOSBW). */
int scalit_build_osbw(scalit_ctx *ctx, double e0, int count, double *de, int npc, int *hwlen);
/* The last window: its size, its grid points (0-based, ascending: WIND - 1)
 * and HW (hwlen x hwlen, column-major: the array saveHW writes,
 * osb.io.h:297-319).  Any output pointer may be null. */
int scalit_get_osbw(scalit_ctx *ctx, int *hwlen, int *ind, double *hw);
/* loadHW (osb.io.h:240-264) then createWH: the window is selected as
 * scalit_build_osbw selects it, HW (count x count, column-major) is taken
 * from the caller instead of being formed, and HWR is inverted. */
int scalit_set_osbw(scalit_ctx *ctx, double e0, int count, double *de, int npc, const double *hw);

/* MYPX (src/iterate/module/osb.px.h:125-219; MPI mosb3.px.h:7-132):
 *   Y = V_sF..V_1 K^-1 V_1^T..V_sF^T X, K^-1 from the sOSB kind,
 * E0 = 0 for npc == TA0, sOSBW%mE0 otherwise.  With SCALIT_TOSBW the
 * window's entries take HWR^-1 (factored once, with the shift given to
 * scalit_build_osbw) and the others 1/(EIG0 - E0). */
int scalit_px(scalit_ctx *ctx, int npc, int nvec, const double *X, double *Y);
int scalit_px_device(scalit_ctx *ctx, int npc, int nvec, const double *dX, double *dY);
int scalit_px_f32_device(scalit_ctx *ctx, int npc, int nvec, const float *dX, float *dY);

/* P*X for one device vector that allocates nothing.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory at call
 * time -- a host code whose device memory is entirely owned by another
 * allocator (a framework's caching pool or a preallocated arena), or a solver
 * loop that must not trigger the implicit device synchronisation of
 * cudaMalloc/cudaFree.  Same operator and kernels as scalit_px_device; its
 * scratch vector is a file-scope device array of 2^20 doubles (8 MiB, held by
 * every GPU that loads this library until the process exits), so grids larger
 * than 1,048,576 points are rejected with SCALIT_EINVAL.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) with the
 * device current; make that first call before any stream capture.  All calls
 * share the one array and it keeps the last call's contents (nothing in it
 * needs to start at zero: every stage overwrites it before reading), so calls
 * that overlap on the GPU -- two streams, or two contexts on one device --
 * race on it.  The looked-up address is cached for the device's primary
 * context: after a cudaDeviceReset in this process the variant must not be
 * called again.  npc other than SCALIT_TA0 / SCALIT_TA1 is SCALIT_EINVAL. */
int scalit_px_noalloc_device(scalit_ctx *ctx, int npc, const double *dX, double *dY);

/* ------------------------------------------------ complex (absorbing) forms --
 * The resonance and CRP jobs: complex vectors (the reference's COMPLEX*16,
 * interleaved real/imaginary, npoints complex values per vector), real H, V
 * and EIG0, complex diagonal.  scalit_set_absorbing loads APP and APR
 * (loadInitData, osb.io.h:18-30,92-112): APR may be null (JOB_RES1/2: APR = 0,
 * AP = APP); otherwise AP = APP + APR (JOB_CRP). */
int scalit_set_absorbing(scalit_ctx *ctx, const double *APP, const double *APR);
/* MYHX_DX (src/iterate/module/osb.hxdx.h:178-240):
 *   Y = (RES - E0 [ntype uses E0] + sign i A) X + sum_level H_level X
 * with sign and A (AP, APP or APR) from the ntype (SCALIT_TA0 .. SCALIT_TMAPR;
 * unknown codes act as TA1, as the reference's default does). */
int scalit_hx_cx(scalit_ctx *ctx, int ntype, int nvec, const double *X, double *Y);
int scalit_hx_cx_device(scalit_ctx *ctx, int ntype, int nvec, const double *dX, double *dY);
/* The complex-Hamiltonian job (sCX; loadH0 / loadInitData with H0CX, DEPCX,
 * OUTHCX: osb.io.h:49-60, osb.init.h:109-125): complex level matrices H0CX
 * (the concatenation of H0's layout, interleaved COMPLEX*16), complex
 * dependent-level factors DEPCX (may be null) and complex outer per-point
 * matrices OUTHCX (sNDVR; else null), real RES.  Loads their real parts as
 * scalit_load does and keeps the imaginary parts, after which every complex
 * form (scalit_hx_cx, QMR_CX, the complex PISTs, the CRP) applies MYHX_CX
 * (osb.hxcx.h:191-261, H1X_XYZ_CX / H1X_DEP_CX / H3X_CX: hpx_cx.f90:6-34,
 * matrix_cx.f90:97-208): Y = D X + sum_level H_level X with complex H_level.
 * The OSB preconditioner is built from the real parts (the reference's
 * HosbDiagDX rotates the stacked real and imaginary parts of HOSBCX; not
 * provided), which changes the inner solves' convergence, not their
 * solutions.  The real entry points (scalit_hx, scalit_qmr, scalit_pist) see
 * the real parts. */
int scalit_load_cx(scalit_ctx *ctx, const double *H0CX, const double *RES, const double *DEPCX,
                   const double *OUTHCX);
/* MYPX_DX (src/iterate/module/osb.mypxdx.h): V^T of every level, the kernel
 * 1/(EIG0 - E0 + sign i A) (E0 = 0 for TA0, TAAP0, TMAP0; TOSBD1 clamps
 * |EIG0 - E0| <= DE to +-DE; TOSBD2 uses alpha + (1 + beta)(EIG0 - E0) on both
 * sides of E0, as the complex reference does), V of every level.  With TOSBW
 * the window's entries take the inverse of HW - E0 +- i A(WIND)
 * (createWH_DXCX, osb.pij.h:63-135; LU on the device, kept per nType and
 * E0), the others the kernel above. */
int scalit_px_cx(scalit_ctx *ctx, int ntype, int nvec, const double *X, double *Y);
int scalit_px_cx_device(scalit_ctx *ctx, int ntype, int nvec, const double *dX, double *dY);
/* QMR_CX (src/iterate/libiterate/qmr/qmrcx.f90:4-175): QMR for the complex
 * symmetric system MYHX_DX(ntype) X = B preconditioned by MYPX_DX(sOSB, ntype),
 * bilinear products X^T Y.  conv selects the convergence test as QMR's ntype
 * does (|1|: |HX - B|/|HX|, |2|: the max of three ratios, else |R|/|B|; X is
 * zeroed when conv <= 0, otherwise X is the start).  *code receives QMR_CX's
 * result (+iterations converged, -iterations not, 0 or -1 on breakdown before
 * the first step) and *res (may be null) RES; the function returns 0 or a
 * library error. */
int scalit_qmr_cx(scalit_ctx *ctx, int conv, int qmrmax, double qmrtol, int ntype, const double *B,
                  double *X, int *code, double *res);
/* Cumulative reaction probability, osbCRP / calOSBCRP
 * (src/iterate/module/osbw.crp.h:6-101): for each of the nenergy energies E
 * (E0 = E during the call; the context's shift is restored afterwards),
 * nm steps of LAN_DX (Hermitian Lanczos with full re-orthogonalisation) on
 * sqrt(APR) (H - E + i AP)^-1 APP (H - E - i AP)^-1 sqrt(APR) from the start
 * vector X0 + e * npoints (interleaved complex; the reference draws it with
 * randMat_CX), each inverse a QMR_CX solve (conv, qmrmax, qmrtol) with the
 * preconditioner's absorbing term when sap != 0 (sAP; otherwise its real
 * kernel, sPC = TA1).  crp[e] = 4 times the sum of the Lanczos eigenvalues
 * (the tridiagonal's trace), 0 when the Lanczos breaks down. */
int scalit_crp(scalit_ctx *ctx, int nenergy, const double *energies, int nm, int qmrmax, double qmrtol,
               int conv, int sap, const double *X0, double *crp);
/* PIST for the complex symmetric operator, PIST_CONV_SX
 * (src/iterate/libiterate/pist/pist_sx.f90:4-96, pistHij_sx.f90:62-118,
 * orth/gsorth_sx.f90:47-72): the Krylov basis of the QMR_CX solves
 * (ls_ntype for H, ls_px_ntype for P, conv / qmrmax / qmrtol; the context's
 * shift is their E0) in the bilinear product, HMAT = VJ^T H0 VJ with H0 =
 * MYHX_DX(h0_ntype), its eigenvalues by cuSOLVER's general eigensolver (ZGEEV
 * in the reference), the m nearest e0 by the real part, converged when the
 * change of |lambda|^2 is <= etol.  eig receives m interleaved complex values
 * in ascending real part, *status PIST's result (+cnt, -cnt, 0 for bad
 * parameters).  ntype > 0 returns SCALIT_EUNSUP: the reference's call of
 * getSepMax_CX there passes mismatched arguments.  conjugate != 0 runs
 * PIST_CONV_CX (pist/pist_cx.f90) instead: the same steps in the conjugated
 * product (MGS_ORTH_CX, HMAT = VJ^H H0 VJ), the driver's JOB_RES2. */
int scalit_pist_cx(scalit_ctx *ctx, double e0, double etol, int ntype, int conjugate, const double *X0,
                   int startcnt, int stepcnt, int stepeig, int m, int m_max, int h0_ntype, int ls_ntype,
                   int ls_px_ntype, int conv, int qmrmax, double qmrtol, double *eig, double *res, int *status);

/* ------------------------------------------------------------------ QMR ---
 * OSB_QMR -> QMR / QMR_MPI (src/iterate/module/osbw.qmr.h:13-23,
 * src/iterate/libiterate/qmr/qmr.f90:5-175,
 * src/iterate/libiterate_mpi/qmr/qmr_mpi.f90:4-263) on HX = (H-E0)X and
 * PX = MYPX(sOSB, TA1), with x0 = 0 when ntype <= 0.  ntype selects the
 * convergence test: |1| uses |HX - B|/|HX| (one extra H*X per iteration),
 * |2| the max of three ratios, otherwise |R|/|B|.  Returns the reference's
 * QMR_MPI code; *res receives RES and *iters (may be NULL) the iteration
 * count.  precision = SCALIT_PREC_FP64, SCALIT_PREC_FP32 (vectors, H*X
 * and P*X in FP32, reductions accumulated in FP64; B and X stay FP64 at the
 * boundary) or SCALIT_PREC_FP32_REFINED: FP32 solves of the current FP64
 * residual r = B - (H - E0) X added to X (at most 5 rounds, each solved to
 * max(1e-4, qmrtol |B - r| / |r|) and capped by the iterations left), until
 * |r| <= qmrtol |B - r| -- the type -1 measure in FP64 -- so a tolerance the
 * FP32 recurrence cannot attain is still reached (no counterpart in the
 * reference, an extension of QMR for the mixed-precision solve); the code is
 * the total iteration count, negative when the tolerance was not reached. */
int scalit_qmr(scalit_ctx *ctx, int ntype, int qmrmax, double qmrtol, int precision,
               const double *B, double *X, double *res, int *iters);
int scalit_qmr_device(scalit_ctx *ctx, int ntype, int qmrmax, double qmrtol, int precision,
                      const double *dB, double *dX, double *res, int *iters);
/* The same two solves with QMR's code in *code and 0 (or a library error) as
 * the result: a not-converged solve of more than 100 iterations returns
 * -iterations <= -101 from scalit_qmr, which a caller cannot tell from a
 * library error; these keep the two apart. */
int scalit_qmr_ex(scalit_ctx *ctx, int ntype, int qmrmax, double qmrtol, int precision, const double *B,
                  double *X, int *code, double *res, int *iters);
int scalit_qmr_device_ex(scalit_ctx *ctx, int ntype, int qmrmax, double qmrtol, int precision,
                         const double *dB, double *dX, int *code, double *res, int *iters);

/* ----------------------------------------------- shifts and batches -----
 * No reference counterpart: the reference solves one system per QMR call
 * (qmr.f90:5-175).  QMR on nrhs right-hand sides at once: column v of dB / dX
 * (npoints x nrhs, device, FP64) solves (H - shifts[v]) x = b with the
 * preconditioner's kernel shifted to shifts[v] (the ctx's sOSB kind, TA1);
 * all columns advance in lockstep through batched H*X / P*X launches, each
 * with its own recurrence and stopping test (ntype, qmrmax, qmrtol as in
 * scalit_qmr; precision SCALIT_PREC_FP32 runs the vectors and operators in
 * FP32).  codes[v] (may be NULL) receives QMR_MPI's status of column v and
 * res[v] (may be NULL) its final residual measure. */
int scalit_qmr_shifts_device(scalit_ctx *ctx, int nrhs, const double *shifts, int ntype, int qmrmax,
                             double qmrtol, int precision, const double *dB, double *dX, int *codes,
                             double *res);
/* The same for nprob independent problems on one GPU (each context loaded,
 * preconditioned and with its own stream), advanced together by one CUDA graph
 * with a branch per problem.  shifts, codes, res: nprob x nrhs (problem-major);
 * dB[p], dX[p]: problem p's device arrays.  *seconds (may be NULL) receives the
 * device time of the iterations. */
int scalit_qmr_shifts_batch(scalit_ctx *const *ctxs, int nprob, int nrhs, const double *shifts, int ntype,
                            int qmrmax, double qmrtol, int precision, const double *const *dB,
                            double *const *dX, int *codes, double *res, double *seconds);

/* ----------------------------------------------------------------- PIST ---
 * OSB_PISTCONV -> PIST_CONV / PIST_CONV_MPI
 * (src/iterate/module/osbw.pistconv.h:16-50, setPISTConvParam :303-333;
 * src/iterate/libiterate/pist/pist.f90:7-98, pistHij.f90:70-125;
 * src/iterate/libiterate_mpi/pist/pist_mpi.f90:11-191, pistHij_mpi.f90:83-190).
 * Krylov vectors from inexact QMR solves of (H-E0) w = v_J, full
 * re-orthogonalisation in FP64, HMAT = V^T H V in FP64, Ritz values of HMAT
 * on the device, window of m values nearest e0, convergence by the largest
 * change (ntype <= 0) or separation (ntype > 0). */
typedef struct {
    double e0;        /* sConv%mE0: window centre                        */
    double etol;      /* sConv%mTol                                      */
    int ntype;        /* sPISTConvType (0: getDiffMax)                   */
    int startcnt;     /* pistStart                                       */
    int stepcnt;      /* pistStep                                        */
    int stepeig;      /* pistEigStep                                     */
    int m;            /* sConv%mNum: number of eigenvalues               */
    int m_max;        /* pistNMax                                        */
    int qmr_ntype;    /* sQMRConvType (-1)                               */
    int qmr_max;      /* sQMR%mMax                                       */
    double qmr_tol;   /* sQMR%mTol                                       */
    int precision;    /* SCALIT_PREC_* of the QMR inner solves           */
    int verbose;      /* print the reference's per-step lines to stdout  */
    int orth;         /* 0: one modified Gram-Schmidt pass in the        */
                      /*    reference's order (MGS_ORTH);                */
                      /* 1: classical Gram-Schmidt twice (default: keeps */
                      /*    the basis orthonormal over long runs);       */
                      /* 2: as 1 with the first pass in FP32 against an  */
                      /*    FP32 copy of the basis (N x m_max floats);   */
                      /*    the second pass projects in FP64 and applies */
                      /*    its (tiny) coefficients, split into two FP32 */
                      /*    parts, over the FP32 copy: orthonormal to    */
                      /*    FP64 round-off                               */
                      /* 3: as 2 with the first pass's update over the   */
                      /*    FP64 basis: the FP32 copy's rounding adds    */
                      /*    ~6e-8 |c| outside the basis' span in mode 2, */
                      /*    which sets a residual floor of ~3e-8 Eh      */
                      /*    (use 3 with a residual target)               */
} scalit_pist_params;

typedef struct {
    int krylov;        /* final cnt_high                                 */
    int qmr_total;     /* sum of QMR iterations (num3)                   */
    int qmr_solves;    /* number of QMR solves                           */
    int checks;        /* number of Ritz checks                          */
    double t_qmr;      /* seconds in QMR solves                          */
    double t_orth;     /* seconds in re-orthogonalisation                */
    double t_hmat;     /* seconds building HMAT columns                  */
    double t_ritz;     /* seconds waiting for the Ritz eigen-solves      */
    double t_resid;    /* seconds in the final Ritz-vector residual check */
} scalit_pist_info;

/* Fill params from the input-file values the way setPISTConvParam does:
 * conv = (mE0, mTol, mStart, mStep, mMax, mNum, mGap), qmr = (mMax, mTol). */
void scalit_pist_default_params(scalit_pist_params *p, int m0, double conv_e0, double conv_tol,
                                int conv_start, int conv_step, int conv_max, int conv_gap,
                                int qmr_max, double qmr_tol);
/* x0: npoints start vector (host).  eig: m values ascending.  info may be NULL. */
int scalit_pist(scalit_ctx *ctx, const scalit_pist_params *p, const double *x0, double *eig,
                double *res, scalit_pist_info *info);

/* ------------------------------------------------ Differentiation -------
 * Adjoint of Y = MYHX(ntype) X for one vector: given the cotangent Ybar,
 *   Xbar = H^T Ybar (the shifted operator with transposed level matrices),
 *   Vbar = Ybar .* X (gradient with respect to the potential grid RES),
 *   H0bar(level l) = sum over the other levels of s_l Ybar (x) X
 *     (gradient with respect to each level matrix, laid out like H0; s_l is
 *     the DEP factor of a dependent level).
 * Any output pointer may be NULL.  No counterpart in the reference (which
 * has no derivatives); it extends MYHX (osb.hx.h:71-110). */
int scalit_hx_adjoint(scalit_ctx *ctx, int ntype, const double *X, const double *Ybar, double *Xbar,
                      double *Vbar, double *H0bar);
int scalit_hx_adjoint_device(scalit_ctx *ctx, int ntype, const double *dX, const double *dYbar,
                             double *dXbar, double *dVbar, double *dH0bar);
int scalit_hx_adjoint_f32_device(scalit_ctx *ctx, int ntype, const float *dX, const float *dYbar,
                                 float *dXbar, float *dVbar, float *dH0bar);
/* Hellmann-Feynman gradients dE_k/dp_j = <psi_k| dV/dp_j |psi_k> for m
 * normalised eigenvectors psi (m x npoints) and np potential derivatives
 * dvdp (np x npoints); grad receives m x np values (row k, column j). */
int scalit_hf_gradients(scalit_ctx *ctx, int m, const double *psi, int np, const double *dvdp,
                        double *grad);
/* PIST as scalit_pist, also returning the m Ritz vectors of the converged
 * levels (m x npoints, host, same order as eig): psi_k = V_basis y_k with y_k
 * the eigenvector of HMAT (DSYEV 'V' in place of the reference's 'N'). */
int scalit_pist_vectors(scalit_ctx *ctx, const scalit_pist_params *p, const double *x0, double *eig,
                        double *res, scalit_pist_info *info, double *vectors);
/* PIST as scalit_pist, followed by the final FP64 residual check of the
 * converged levels: resid[k] = |H psi_k - eig_k psi_k|_2 for the normalised
 * Ritz vector psi_k (H without shift, one batched FP64 H*X on the device).
 * The reference reports no residuals (pist.f90 returns eigenvalues only). */
int scalit_pist_residuals(scalit_ctx *ctx, const scalit_pist_params *p, const double *x0, double *eig,
                          double *res, scalit_pist_info *info, double *resid);

/* PIST with a residual-based continuation, no counterpart in the reference
 * (whose stopping test is the eigenvalue change alone, getDiffMax,
 * util.f90:84-100): once that test passes, the FP64 residuals
 * |H psi_k - theta_k psi_k|_2 of the window's Ritz pairs are checked, and
 * while one is above resid_tol (Eh) the Krylov basis grows by
 * max(stepcnt, K/20) vectors and the check repeats, at most max_steps times
 * and up to m_max vectors.  The residual floor is set by the inner solves'
 * accuracy: a 1e-8 Eh target wants p->qmr_tol <= 1e-6, in FP64 or
 * SCALIT_PREC_FP32_REFINED.  eig receives the window's Ritz values of the
 * final basis (ascending), resid their residuals, vectors (m x npoints, may be
 * NULL) the Ritz vectors, *steps (may be NULL) the number of extensions; the
 * result is the final Krylov size (or the usual failure codes).
 * info->t_resid includes the checks and the extensions' solves. */
int scalit_pist_refined(scalit_ctx *ctx, const scalit_pist_params *p, const double *x0, double *eig,
                        double *res, scalit_pist_info *info, double resid_tol, int max_steps,
                        double *resid, double *vectors, int *steps);

/* PIST followed by the output of PISTF_CONV (src/iterate/libiterate/pist/pistf.f90:98-104):
 * on success *cnt receives the final Krylov size, ritz the cnt Ritz values of
 * the last Rayleigh-Ritz step, hmat HMAT(1:cnt, 1:cnt) column-major and vj the
 * basis VJ(1:N, 1:cnt).  Size the buffers for p->m_max (ritz: m_max, hmat:
 * m_max^2, vj: npoints * m_max).  Any of ritz/hmat/vj may be NULL. */
int scalit_pist_basis(scalit_ctx *ctx, const scalit_pist_params *p, const double *x0, double *eig,
                      double *res, scalit_pist_info *info, int *cnt, double *ritz, double *hmat,
                      double *vj);

/* -------------------------------------------- Fortran drop-in symbols -----
 * The external routines the reference's modules call, with gfortran naming
 * (lower case, trailing underscore) and every argument by reference.  They
 * operate on caller HOST arrays and run on the GPU of the default context
 * (device 0 unless scalit_fortran_device_ was called).  Operator callbacks:
 * when qmr_/qmr_mpi_/pist_conv_/pist_conv_mpi_ receive this library's own
 * scalit_ehx_/scalit_hx0_/scalit_epx_/scalit_osb_qmr_ they run
 * device-resident on the context made by scalit_fortran_init_; any other
 * callback is called with host vectors. */

/* H1X_XYZ (src/iterate/libiterate/hpx/hpx.f90:5-18) and
 * H1X_XYZ_Seq (src/iterate/libiterate_mpi/hpxseq/hpx_seq.f90:7-32). */
void h1x_xyz_(const int *nin, const int *nout, const int *blk, const double *H1,
              const double *X, double *Y);
void h1x_xyz_seq_(const int *nin, const int *nout, const int *blk, const double *H1,
                  const double *X, double *Y);
/* H1TX_XYZ_Seq (hpx_seq.f90:36-60). */
void h1tx_xyz_seq_(const int *nin, const int *nout, const int *blk, const double *H1,
                   const double *X, double *Y);
/* H1X_DEP (hpx.f90:21-35) and H2X_DEP_Seq (hpx_seq.f90:67-92). */
void h1x_dep_(const int *nin, const int *nout, const int *blk, const double *H1,
              const double *CORX, const double *X, double *Y);
void h2x_dep_seq_(const int *nin, const int *nout, const int *blk, const double *H1,
                  const double *DEPX, const double *X, double *Y);
/* H3X_Out_Seq (hpx_seq.f90:129-154): per-point outer matrices. */
void h3x_out_seq_(const int *nin, const int *nout, const int *blk, const double *OUTH,
                  const double *X, double *Y);
/* VX / VTX (hpx.f90:40-73) and VX_Seq / VTX_Seq (hpx_seq.f90:192-254), in place. */
void vx_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X);
void vtx_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X);
void vx_seq_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X);
void vtx_seq_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X);
/* HosbDiag (src/iterate/libiterate/diag/hosbdiag.f90:5-75) and
 * HosbDiag_Seq (src/iterate/libiterate_mpi/diagseq/hosbdiag_seq.f90:5-90). */
void hosbdiag_(const int *bjmax, const double *bjtol, const int *blk, const int *mak,
               const int *ndk, double *HOSB, double *VOSB, double *EIGVAL);
void hosbdiag_seq_(const int *bjmax, const double *bjtol, const int *blk, const int *mak,
                   const int *ndk, double *HOSB, double *VOSB, double *EIGVAL, const int *id);
/* HOSBDIAG_MPI (src/iterate/libiterate_mpi/diagmpi/hosbdiag_mpi.f90:5-96) on
 * one rank: comm and id are ignored (the whole NDK stack is on the device);
 * *ierr = 0 on success, 1 when the device step failed. */
void hosbdiag_mpi_(const int *comm, const int *bjmax, const double *bjtol, const int *blk,
                   const int *mak, const int *ndk, double *HOSB, double *VOSB, double *RES,
                   int *ierr, const int *id);
/* MJACOBI (src/iterate/libiterate/diag/jacobi.f90:2-83): one joint Jacobi
 * rotation of the (P, Q) plane (1-based) of HOUT(NIN, NOUT, NOUT), in place;
 * returns the rotation angle X.  The sums A, B, C and the rotation run on the
 * device; the angle is taken on the host with the reference's branches. */
double mjacobi_(const int *p, const int *q, const int *nout, const int *nin, double *HOUT);
/* NORM_MPI / DOTPROD_MPI (src/libutil/parallel/p_base/vector_mpi.f90:8-27,110-124);
 * comm is ignored: one device holds the whole vector. */
double norm_mpi_(const int *comm, const int *nin, const double *X, int *ierr);
double dotprod_mpi_(const int *comm, const int *nin, const double *X, const double *Y,
                    int *ierr);
/* MGS_ORTH (src/iterate/libiterate/orth/gsorth.f90:42-72) and MGS_ORTH_MPI
 * (src/iterate/libiterate_mpi/orth/gsorth_mpi.f90:45-76): returns a Fortran
 * logical (1 = .true.). */
int mgs_orth_(const int *n, const double *WJ, const int *m, double *VJ);
int mgs_orth_mpi_(const int *n, const double *WJ, const int *m, double *VJ, int *ierr);
/* QMR (qmr.f90:5) and QMR_MPI (qmr_mpi.f90:4). */
typedef void (*scalit_fortran_op)(const int *n, const double *x, double *y);
typedef int (*scalit_fortran_linsolv)(const int *n, const double *b, double *x, double *res);
int qmr_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n,
         const double *B, scalit_fortran_op hx, scalit_fortran_op px, double *X, double *RES);
/* QMR_CX (src/iterate/libiterate/qmr/qmrcx.f90:4-175) and PIST_CONV_SX
 * (src/iterate/libiterate/pist/pist_sx.f90:4-96), the complex library's
 * externals: B, X, EIG are COMPLEX*16 arrays (interleaved) and the callbacks
 * receive them as such; the recurrences run on the GPU.  QMR_CX returns its
 * code (-10 when the library fails, with a message on stderr); PIST_CONV_SX
 * its status (0 for bad parameters and for ntype > 0, whose result the
 * reference leaves undefined). */
int qmr_cx_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n, const double *B,
            scalit_fortran_op hx, scalit_fortran_op px, double *X, double *RES);
int pist_conv_sx_(const double *e0, const double *etol, const int *ntype, const int *n, const double *X,
                  const int *startcnt, const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
                  scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG, double *RES);
/* PIST_CONV_CX (src/iterate/libiterate/pist/pist_cx.f90): PIST_CONV_SX in the
 * conjugated product (MGS_ORTH_CX, HMAT = VJ^H H0 VJ). */
int pist_conv_cx_(const double *e0, const double *etol, const int *ntype, const int *n, const double *X,
                  const int *startcnt, const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
                  scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG, double *RES);
int qmr_mpi_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n,
             const double *B, scalit_fortran_op hx, scalit_fortran_op px, double *X,
             double *RES, const int *myid);
/* PIST_CONV (pist.f90:7) and PIST_CONV_MPI (pist_mpi.f90:11). */
int pist_conv_(const double *e0, const double *etol, const int *ntype, const int *n,
               const double *X, const int *startcnt, const int *stepcnt, const int *stepeig,
               const int *m, const int *m_max, scalit_fortran_op h0x,
               scalit_fortran_linsolv linsolv, double *EIG, double *RES);
/* pistH0 (src/iterate/libiterate/pist/pistHij.f90:70-125) and pistH0_MPI
 * (src/iterate/libiterate_mpi/pist/pistHij_mpi.f90:83-190): the Krylov
 * vectors m_low..m_high (from LinSolv and one modified Gram-Schmidt pass) and
 * their HMAT columns, on the caller's VJ(N, M_HIGH) and HMAT(M_MAX, M_HIGH).
 * Returns m_high, LinSolv's code (<= 0) when it failed, -J when the
 * orthogonalisation failed at J, 0 for bad sizes.  *num2 (MPI form) receives
 * the sum of LinSolv's codes.  Given scalit_hx0_ and scalit_osb_qmr_ the
 * operators run on the module state without host staging. */
int pisth0_(const int *n, const double *X, const int *m_max, const int *m_low, const int *m_high,
            scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *VJ, double *HMAT);
int pisth0_mpi_(const int *myid, const int *rootid, const int *n, const double *X, const int *m_max,
                const int *m_low, const int *m_high, scalit_fortran_op h0x,
                scalit_fortran_linsolv linsolv, double *VJ, double *HMAT, int *num2);
int pist_conv_mpi_(const int *myid, const int *rootid, const double *e0, const double *etol,
                   const int *ntype, const int *n, const double *X, const int *startcnt,
                   const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
                   scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG,
                   double *RES);

/* Module-state seam for the drivers: replaces loadInitData + progDiag and
 * supplies the operator callbacks HX0 (TA0), EHX (TA1), EPX (MYPX TA1) and
 * OSB_QMR (sQMRConvType, sQMR%mMax, sQMR%mTol).  A trailing IERR argument
 * passed by the MPI library is tolerated. */
void scalit_fortran_device_(const int *device);
void scalit_fortran_init_(const int *sf, const int *sn, const int *sdep, const double *H0,
                          const double *RES, const double *DEP, const double *e0, int *ierr);
void scalit_fortran_precond_(const int *sosb, const double *de, const double *beta,
                             const int *bjmax, const double *bjtol, int *ierr);
/* initOSBW (osb.osbw.h:2-50) on the module state, after scalit_fortran_precond_
 * with sOSB = 4 (which builds the preconditioner only): the window of
 * sOSBW%mCnt states around sOSBW%mE0 from the width sOSBW%mDE (updated in
 * place, as adjustWinSize updates it), factored for sPC = npc; selects TOSBW. */
void scalit_fortran_osbw_(const double *e0, const int *cnt, double *de, const int *npc, int *ierr);
void scalit_fortran_qmr_param_(const int *ntype, const int *qmrmax, const double *qmrtol,
                               const int *precision);
void scalit_fortran_final_(void);
void scalit_hx0_(const int *n, const double *X, double *Y);
void scalit_ehx_(const int *n, const double *X, double *Y);
void scalit_epx_(const int *n, const double *X, double *Y);
int scalit_osb_qmr_(const int *n, const double *B, double *X, double *ERES);

#ifdef __cplusplus
}
#endif
#endif /* SCALIT_GB300_H */
