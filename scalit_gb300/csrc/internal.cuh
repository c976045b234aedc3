// Internal declarations shared by the translation units of libscalit_gb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/scalit_gb300.h"

typedef long long i64;

namespace sc {

// ------------------------------------------------------------------ errors --
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define SC_CUDA(call)                                                         \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return sc::cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

#define SC_CHECK_LAUNCH() SC_CUDA(cudaGetLastError())

// ------------------------------------------------------------------ layout --
// calOSB (src/iterate/module/osb.init.h:2-49): per-level dimensions and the
// start offsets of each level inside the concatenated H0 / DEP / VOSB arrays.
struct Layout {
    int nlev = 0;
    int n[SCALIT_FMAX] = {};
    int dep[SCALIT_FMAX] = {};
    int ndvr = 0;
    i64 dim[SCALIT_FMAX] = {};  // myDim: product of the faster levels' sizes
    i64 blk[SCALIT_FMAX] = {};  // myBlk: product of the slower levels' sizes
    i64 h0s[SCALIT_FMAX] = {};  // start of level l in H0
    i64 deps[SCALIT_FMAX] = {}; // start of level l in DEP
    i64 vs[SCALIT_FMAX] = {};   // start of level l in VOSB
    i64 N = 0, h0len = 0, deplen = 0, vlen = 0, outhlen = 0;
    void compute();
};

// Device vector with FP64 master and optional FP32 shadow.
template <class T> struct DevBuf {
    T *p = nullptr;
    i64 n = 0;
};

}  // namespace sc

// Tensor-core plan of one level: the level matrix cut into 7 BF16 digit planes.
struct TcLevelData {
    uint16_t *dig = nullptr;   // [ntiles][KS][7][NT x 16] BF16 bits
    int *exps = nullptr;       // [ntiles * NT] column exponents
    float *cscale = nullptr;   // [NT] inverse column scales (FP16 planes)
    int NT = 0, ntiles = 0, KS = 0, usable = 0;
};

// The opaque context of the C ABI.
struct scalit_ctx {
    sc::Layout L;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;   // the context's own stream while a caller's is set
    cudaStream_t s_in = nullptr, s_out = nullptr;   // host<->device copy streams
    cudaEvent_t ev[6] = {};                          // copy/compute ordering events
    // FP64 operator data (module globals H0/RES/DEP/OUTH/EIG0/VOSB in the reference)
    double *H0 = nullptr, *RES = nullptr, *DEP = nullptr, *OUTH = nullptr;
    double *EIG0 = nullptr, *VOSB = nullptr;
    // FP32 shadows for the mixed-precision inner solves
    float *H0f = nullptr, *RESf = nullptr, *DEPf = nullptr, *OUTHf = nullptr;
    float *EIG0f = nullptr, *VOSBf = nullptr;
    bool loaded = false, osb_built = false;
    double E0 = 0.0;
    int osb_kind = SCALIT_TOSB;
    double osb_de = 0.0, osb_beta = 0.0;
    // OSBW window (sOSB = TOSBW): its grid points, HW (column-major), the
    // inverse of HW - shift I in FP64 and FP32 (both triangles), and room for
    // the gathered window entries of one P*X.  osbw_valid turns false when
    // the preconditioner the window was made from changes.
    int osbw_len = 0;
    bool osbw_valid = false;
    int *osbw_ind = nullptr;
    double *osbw_hw = nullptr, *osbw_inv = nullptr;
    float *osbw_invf = nullptr;
    void *osbw_wy = nullptr;
    double osbw_e0 = 0.0, osbw_de = 0.0;
    long long osbw_serial = 0;            // counts the windows made
    // the complex window matrix's inverse for one nType and E0 (interleaved
    // complex, hwlen x hwlen) and room for one P*X's gathered complex entries
    double *osbw_cxinv = nullptr, *osbw_cxw = nullptr;
    int osbw_cx_ntype = -1;
    double osbw_cx_e0 = 0.0;
    long long osbw_cx_serial = -1;
    // absorbing potentials of the complex forms: APP, APR and AP = APP + APR
    double *APP = nullptr, *APR = nullptr, *AP = nullptr;
    // the complex-Hamiltonian job (sCX): imaginary parts of H0CX, DEPCX, OUTHCX
    // (the real parts are H0, DEP, OUTH); cxh is set while they apply
    double *H0i = nullptr, *DEPi = nullptr, *OUTHi = nullptr;
    bool cxh = false;
    // workspace (grown on demand)
    void *work = nullptr;
    size_t work_bytes = 0;
    // reduction scratch: partial sums and a completion counter
    double *red_partial = nullptr;
    unsigned int *red_counter = nullptr;
    double *red_result = nullptr;   // device scalars of the last reductions
    double *h_pinned = nullptr;     // pinned host mirror for scalar readback
    void *cusolver = nullptr;       // cusolverDnHandle_t
    // FP64 H*X engine: SCALIT_FP64_DFMA (FP64 pipe) or SCALIT_FP64_TENSOR (digit-sliced tcgen05)
    int fp64_mode = SCALIT_FP64_TENSOR;
    // FP32 engine: SCALIT_FP32_SIMT (CUDA cores), SCALIT_FP32_TENSOR (split-BF16 x3)
    // or SCALIT_FP32_TENSOR_PX (split-BF16 x3 for the preconditioner's rotations only)
    int fp32_mode = SCALIT_FP32_SIMT;
    // precision of the preconditioner build's one-matrix Jacobi sweeps
    // (SCALIT_PREC_FP64, or SCALIT_PREC_FP32 for FP32 inner solves)
    int build_prec = SCALIT_PREC_FP64;
    // storage of the level-1 preconditioner matrices for the FP32 P*X: 32
    // (VOSBf) or 16 (an FP16 copy, VOSBh, made by px_half_prepare)
    int px_bits = 32;
    void *VOSBh = nullptr;
    TcLevelData tc32[SCALIT_FMAX];           // hi/lo planes of the level matrices
    TcLevelData pxtc32[SCALIT_FMAX][2];      // of the preconditioner's rotations [VX, VTX]
    TcLevelData tc[SCALIT_FMAX];
    // digit planes of the preconditioner's rotations, levels >= 2: [level][VX, VTX]
    TcLevelData pxtc[SCALIT_FMAX][2];
    // FP16 hi/lo planes of the level matrices with their column scales
    // (SCALIT_FP32_TENSOR16) and the per-vector scale slots of one launch
    TcLevelData tc16[SCALIT_FMAX];
    unsigned *xmax = nullptr;
    int *rexp = nullptr;                    // row exponents of the persistent FP64 engine's levels
    i64 rexp_off[SCALIT_FMAX] = {};
    int *tc_err = nullptr;
    // Measurement aid: when set, hx_batch records lev_ev[l] before level l's
    // launch and lev_ev[nlev] after the last (scalit_hx_level_times).
    cudaEvent_t *lev_ev = nullptr;
    // Captured QMR iteration batches (one per precision); `gen` changes whenever
    // anything baked into the captured launches changes (shift, preconditioner,
    // engine, workspace), which invalidates them.
    long long gen = 0;
    // CUDA-core GEMM tile per [FP64, FP32][level][one vector, many]: -1 untuned
    signed char tile_pick[2][SCALIT_FMAX][2];
    // wall seconds per level of the last preconditioner build
    double build_s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    struct QmrGraph { cudaGraphExec_t exec = nullptr; long long gen = -1; int ntype = 0; i64 n = 0; void *work = nullptr; int nrhs = 0; } qg[2];
};

namespace sc {

// Workspace: returns a device pointer with at least `bytes` bytes.
int work_get(scalit_ctx *c, size_t bytes, void **out);

// ----------------------------------------------------- contraction kernels --
// C[m, n] (+)= rowscale[m % Mi] * sum_k A[m, k] * B[k, n]  with
//   A(m,k) = A + moff(m) + k*a_sk,  B(k,n) = B + k*b_sk + n*b_sn,
//   C(m,n) = C + moff(m) + n*c_sn,  moff(m) = (m % Mi)*s1 + (m / Mi)*s2,
// per batch z: A += z*a_sz, B += z*b_sz, C += z*c_sz.
// Epilogue: out = (accumulate ? C : 0) + alpha*scale*acc
//           + (diagV ? (diagV[p] - shift) * diagX[p] : 0) with p = C offset.
template <class T> struct GemmArgs {
    int M, N, K, batch;
    i64 Mi, s1, s2;          // A's row offset (m % Mi) s1 + (m / Mi) s2
    i64 c_s1 = -1, c_s2 = -1; // C's row strides; -1: the same as A's
    const T *A; i64 a_sk, a_sz;
    const T *B; i64 b_sk, b_sn, b_sz;
    T *C; i64 c_sn, c_sz;
    const T *rowscale;     // may be null
    int accumulate;
    T alpha;
    const T *diagV;        // may be null
    const T *diagX;
    i64 dx_sz;             // batch stride of diagX
    T shift;
    const T *shiftv = nullptr;   // per-batch shifts (batch index z), overriding shift
    int tile = -1;               // 0: big tile, 1: small tile, -1: by the CTA count
    int b_mod = 0;               // > 0: B of batch z is B + (z % b_mod) b_sz
    const int *vgate = nullptr;  // per-vector stop flags: batch z is skipped when
    int vgate_stride = 0;        //   vgate[(z / vgate_div) * vgate_stride] != 0
    int vgate_div = 1;
    const int *gate;       // if non-null and *gate != 0 the kernel does nothing
};

template <class T> int launch_gemm(const GemmArgs<T> &g, cudaStream_t s);

// One level of MYHX: out (+)= H_level X (dependent levels scaled by DEP).
template <class T>
int level_apply(const scalit_ctx *c, int level, const T *H0, const T *DEP, const T *OUTH,
                const T *X, T *Y, int accumulate, const T *diagV, T shift, T alpha,
                const int *gate, cudaStream_t s, int nvec = 1, const T *shiftv = nullptr,
                const int *vgate = nullptr, int vstride = 0);

// The whole operator on nvec vectors stored back to back (one launch per level).
template <class T>
int hx_batch(const scalit_ctx *c, const T *X, T *Y, int nvec, T shift, T alpha, const int *gate,
             cudaStream_t s, const T *shiftv = nullptr, const int *vgate = nullptr, int vstride = 0);

// Whole operator for one vector: Y = alpha * ((V - shift) X + sum_l H_l X).
template <class T>
int hx_vec(const scalit_ctx *c, const T *X, T *Y, T shift, T alpha, const int *gate,
           cudaStream_t s);

// Whole preconditioner for one vector: Y = alpha * V K^-1 V^T X.  tmp: N elements.
template <class T>
int px_vec(const scalit_ctx *c, int npc, const T *X, T *Y, T *tmp, T alpha, const int *gate,
           cudaStream_t s);
// P*X of nvec vectors (stride npoints), vector v with kernel shift e0v[v] (device, TA1)
template <class T>
int px_multi(const scalit_ctx *c, const T *X, T *Y, T *tmp, int nvec, const double *e0v, const int *gate,
             cudaStream_t s, const int *vgate = nullptr, int vstride = 0);

// Generic per-level rotation (VX / VTX) on device arrays, out of place.
template <class T>
int level_rotate(int nin, int nout, int blk, const T *V, const T *X, T *Y, int transpose,
                 const int *gate, cudaStream_t s);

// -------------------------------------------------------- differentiation --
template <class T>
int hx_adjoint(scalit_ctx *c, int ntype, const T *X, const T *Ybar, T *Xbar, T *Vbar, T *Hbar, cudaStream_t s);
int hf_gradients(scalit_ctx *c, int m, const double *psi, int np, const double *dvdp, double *grad_dev);

// ------------------------------------------------------- tensor-core FP64 --
int gemm_autotune(scalit_ctx *c, int nvec_many);
int tc32_prepare(scalit_ctx *c, bool rotations);
void tc32_free(scalit_ctx *c, bool levels, bool rotations);
bool tc32_usable(const scalit_ctx *c, int level);
bool tc32_px_usable(const scalit_ctx *c, int level);
int tc32_level_apply(const scalit_ctx *c, int level, const float *X, float *Y, int accumulate, const float *diagV,
                     float shift, float alpha, const int *gate, cudaStream_t s, int nvec,
                     const float *shiftv = nullptr, const int *vgate = nullptr, int vstride = 0);
int tc32_rot_apply(const scalit_ctx *c, int level, int transpose, const float *X, float *Y, const int *gate,
                   cudaStream_t s, int nvec = 1, const int *vgate = nullptr, int vstride = 0);
int tma_encode(CUtensorMap *map, const void *base, bool f64, int rank, const cuuint64_t *dims,
               const cuuint64_t *strides, const cuuint32_t *box, CUtensorMapSwizzle swz);
int tc16_prepare(scalit_ctx *c);
int tc64p_prepare(scalit_ctx *c);
bool tc64p_usable(const scalit_ctx *c, int level);
int tc64p_vectors_max();
int tc64p_rowexp(const scalit_ctx *c, int level, const double *X, int nvec, const int *gate, cudaStream_t s,
                 const int *vgate = nullptr, int vstride = 0);
int tc64p_level_apply(const scalit_ctx *c, int level, const double *X, double *Y, int accumulate,
                      const double *diagV, double shift, double alpha, const int *gate, cudaStream_t s, int nvec,
                      const double *shiftv = nullptr, const int *vgate = nullptr, int vstride = 0);
void tc16_free(scalit_ctx *c);
bool tc32p_usable(const scalit_ctx *c, int level, bool f16, bool diag = false);
int tc16_scales(const scalit_ctx *c, const float *X, int nvec, const int *gate, cudaStream_t s,
                const int *vgate = nullptr, int vstride = 0);
int tc32p_level_apply(const scalit_ctx *c, int level, bool f16, const float *X, float *Y, int accumulate,
                      const float *diagV, float shift, float alpha, const int *gate, cudaStream_t s, int nvec,
                      const float *shiftv = nullptr, const int *vgate = nullptr, int vstride = 0);
int tc_prepare(scalit_ctx *c);
int tc_prepare_px(scalit_ctx *c);
void tc_free_px(scalit_ctx *c);
bool tc_px_usable(const scalit_ctx *c, int level);
int tc_rot_apply(const scalit_ctx *c, int level, int transpose, const double *X, double *Y, const int *gate,
                 cudaStream_t s);
bool tc_usable(const scalit_ctx *c, int level);
int tc_level_apply(const scalit_ctx *c, int level, const double *X, double *Y, int accumulate,
                   const double *diagV, double shift, double alpha, const int *gate, cudaStream_t s,
                   int nvec, const double *shiftv = nullptr, const int *vgate = nullptr, int vstride = 0);
int tc_check_error(scalit_ctx *c);
int wait_selftest(scalit_ctx *c, double seconds);
int tc_gemm_f64(const scalit_ctx *c, int M, int N, int K, const double *A, i64 lda, const double *B, i64 ldb,
                double *C, i64 ldc, cudaStream_t s);

// VX / VTX of level l (0-based) in FP64, out of place (the real P*X engines).
int px_rotate(const scalit_ctx *c, int l, int transpose, const double *in, double *out, const int *gate,
              cudaStream_t s);

// ---------------------------------------------------------- OSBW window --
// initOSBW for the bound-state job: window width and points, HW (formed, or
// taken from hw_host), the inverse of HW - shift I; selects TOSBW.
int osbw_make(scalit_ctx *c, double e0, int count, double *de, int npc, const double *hw_host, int *hwlen);
void osbw_free(scalit_ctx *c);
void osbw_invalidate(scalit_ctx *c);
// The TOSBW kernel step of P*X in place on Z = V^T X: the window entries
// solved with the window matrix, all others divided by EIG0 - e0, times alpha.
template <class T>
int osbw_window_apply(const scalit_ctx *c, T *Z, const T *EIG, double e0, T alpha, const int *gate, cudaStream_t s);

// ------------------------------------------------- complex forms (Fortran) --
// QMR_CX / PIST_CONV_SX with a caller's callbacks on interleaved COMPLEX*16
// host arrays (the recurrence on the device of context c, n complex points).
int qmr_cx_host(scalit_ctx *c, i64 n, scalit_fortran_op hx, scalit_fortran_op px, int conv, int qmrmax, double tol,
                const double *B, double *X, int *code, double *res);
int pist_sx_host(scalit_ctx *c, i64 n, double e0, double etol, const double *X0, int startcnt, int stepcnt,
                 int stepeig, int m, int m_max, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *eig,
                 double *res, int *status, int conj);

// ------------------------------------------------------------- OSB build --
int osb_build(scalit_ctx *c, int bjmax, double bjtol, double *stats);
// HosbDiag on a device HOSB(ndk, mak, mak, blk): fills VOSB and EIGVAL.
int mjacobi_device(int P, int Q, int nout, int nin, double *dH, double *dabc, double *angle, cudaStream_t s);
// f32: one-matrix blocks and the stacks of the spread schedule run their
// sweeps in FP32 (a preconditioner built for FP32 inner solves); stacks that
// fit one CTA's shared memory and every other caller run them in FP64.
int px_half_prepare(scalit_ctx *c);
int hosbdiag_device(scalit_ctx *c, int bjmax, double bjtol, int blk, int mak, int ndk,
                    double *HOSB, double *VOSB, double *EIG, double *stats5, cudaStream_t s, bool f32 = false);

// ------------------------------------------------------------ vector ops --
// Deterministic FP64-accumulated dot product; writes the result to *out (device).
template <class T>
int dot_dev(scalit_ctx *c, i64 n, const T *x, const T *y, double *out, cudaStream_t s);
int sync_read_doubles(scalit_ctx *c, const double *dsrc, double *host, int count);

int axpy_dev(i64 n, double a, const double *x, double *y, cudaStream_t s);
int scal_dev(i64 n, double a, double *x, cudaStream_t s);

// Convert between precisions.
int to_f32(const double *x, float *y, i64 n, cudaStream_t s);
int to_f64(const float *x, double *y, i64 n, cudaStream_t s);

// ------------------------------------------------------------------ QMR --
struct QmrResult { int code; double res; int iters; int breakdown; };
// Operator pair of a QMR solve.  hx/px write `out` from `in` on the context's
// stream; device operators honour `gate` (skip when *gate != 0).
template <class T> struct QmrOps {
    virtual ~QmrOps() {}
    virtual int hx(const T *in, T *out, const int *gate) = 0;
    virtual int px(const T *in, T *out, const int *gate) = 0;
    virtual bool host_side() const { return false; }
    virtual void set_scratch(T *) {}   // an N-vector the preconditioner may use
};
template <class T>
int qmr_core(scalit_ctx *c, i64 n, QmrOps<T> &ops, int ntype, int qmrmax, double qmrtol,
             const T *dB, T *dX, QmrResult *out);
// nrhs right-hand sides in lockstep (dB, dX: n x nrhs; out[nrhs])
template <class T>
int qmr_core_n(scalit_ctx *c, i64 n, int nrhs, QmrOps<T> &ops, int ntype, int qmrmax, double qmrtol,
               const T *dB, T *dX, QmrResult *out);
struct QmrState;
const int *qmr_done_flag(const QmrState *st);   // &st->done; state v's flag at + v * qmr_state_stride()
int qmr_state_stride();
// The pieces of one solve, for callers that interleave several solves (one
// CUDA graph over many problems): setup, one iteration's launches, results.
template <class T> struct QmrSolve {
    scalit_ctx *c = nullptr;
    i64 n = 0;
    int nrhs = 1;
    QmrOps<T> *ops = nullptr;
    int ntype = 0, qmrmax = 0;
    double tol = 0.0;
    cudaStream_t s = nullptr;
    T *R = nullptr, *UX = nullptr, *UR = nullptr, *Q = nullptr, *S = nullptr, *V = nullptr, *Z = nullptr;
    T *HX0 = nullptr, *Bw = nullptr, *Xw = nullptr, *Pt = nullptr;
    QmrState *st = nullptr;
    double *partial = nullptr;
    int *alldone = nullptr;
    const int *gate = nullptr;   // the flag that stops the operators (and the host loop)
    int gr = 1, ge = 1;
    int setup(scalit_ctx *ctx, i64 n, int nrhs, QmrOps<T> *ops, int ntype, int qmrmax, double tol,
              const T *B, const T *X, cudaStream_t s);
    int iteration();
    int finish(T *X, QmrResult *out);
};
int qmr_run(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision,
            const double *dB, double *dX, QmrResult *out);

// Shifted right-hand sides and batches of problems (multi.cu).
int shifted_qmr(scalit_ctx *c, int nrhs, const double *shifts, int ntype, int qmrmax, double tol, int precision,
                const double *dB, double *dX, int *codes, double *res);
int batch_qmr(scalit_ctx *const *ctxs, int nprob, int nrhs, const double *shifts, int ntype, int qmrmax,
              double tol, int precision, const double *const *dB, double *const *dX, int *codes, double *res,
              double *seconds);

// ----------------------------------------------------------------- PIST --
struct PistOps {
    virtual ~PistOps() {}
    virtual int h0x(const double *dX, double *dY) = 0;                  // H * x
    virtual int linsolv(const double *dB, double *dX, int *num) = 0;   // (H - E0) x = b
};
struct PistBasisOut { int *cnt = nullptr; double *ritz = nullptr, *hmat = nullptr, *vj = nullptr; };
int pist_core(scalit_ctx *c, i64 N, const scalit_pist_params *p, const double *dx0, PistOps &ops,
              double *eig, double *res, scalit_pist_info *info, double *vectors_host = nullptr,
              const PistBasisOut *basis = nullptr, double *resid = nullptr, double refine_tol = 0.0,
              int refine_max = 0, int *refine_steps = nullptr);
int pisth0_host(scalit_ctx *c, i64 N, const double *X, int m_max, int m_low, int m_high, PistOps &ops, double *VJ,
                double *HMAT, bool mpi, int *num2, int *ret);
int pist_ctx(scalit_ctx *c, const scalit_pist_params *p, const double *dx0, double *eig,
             double *res, scalit_pist_info *info, double *vectors_host = nullptr,
             const PistBasisOut *basis = nullptr, double *resid = nullptr, double refine_tol = 0.0,
             int refine_max = 0, int *refine_steps = nullptr);

}  // namespace sc
