// Complex forms with absorbing potentials (the reference's resonance and CRP
// jobs): MYHX_DX (src/iterate/module/osb.hxdx.h:178-240), MYPX_DX
// (src/iterate/module/osb.mypxdx.h) and QMR_CX
// (src/iterate/libiterate/qmr/qmrcx.f90:4-175).
//
// H, V and EIG0 are real; the vectors and the diagonal are complex.  On the
// device a complex vector is planar (N real parts, then N imaginary parts),
// so the real level products run on both halves as one batch of two vectors
// through the FP64 engines of the real path, and the preconditioner's real
// rotations run on each half.  The C ABI takes and returns the reference's
// interleaved COMPLEX*16 arrays.
#include "internal.cuh"

#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <vector>

namespace sc {

static constexpr int kT = 256;

static int cgrid(i64 n)
{
    const i64 g = (n + kT - 1) / kT;
    return (int)std::max<i64>(1, std::min<i64>(g, 152LL * 16));
}

// nType of the complex forms (osb.data.h:18-22): whether E0 shifts the real
// diagonal, the sign of i A, and which absorbing potential A is.
struct CxTerms {
    bool use_e0;
    int sign;
    const double *A;
};

static int cx_terms(const scalit_ctx *c, int ntype, CxTerms *t)
{
    int which = 0;   // 0: none, 1: AP, 2: APP, 3: APR
    switch (ntype) {
    case SCALIT_TA0: *t = {false, 0, nullptr}; break;
    case SCALIT_TA1: *t = {true, 0, nullptr}; break;
    case SCALIT_TAAP0: *t = {false, 1, nullptr}; which = 1; break;
    case SCALIT_TMAP0: *t = {false, -1, nullptr}; which = 1; break;
    case SCALIT_TAAP: *t = {true, 1, nullptr}; which = 1; break;
    case SCALIT_TAAPP: *t = {true, 1, nullptr}; which = 2; break;
    case SCALIT_TAAPR: *t = {true, 1, nullptr}; which = 3; break;
    case SCALIT_TMAP: *t = {true, -1, nullptr}; which = 1; break;
    case SCALIT_TMAPP: *t = {true, -1, nullptr}; which = 2; break;
    case SCALIT_TMAPR: *t = {true, -1, nullptr}; which = 3; break;
    default: *t = {true, 0, nullptr}; break;   // the reference's default: (H - E0) X
    }
    if (which) {
        if (!c->AP) { set_error("nType %d needs the absorbing potentials: call scalit_set_absorbing", ntype); return SCALIT_ESTATE; }
        t->A = which == 1 ? c->AP : which == 2 ? c->APP : c->APR;
    }
    return 0;
}

// E0 of the preconditioner's kernel (MYPX_DX: 0 for TA0, TAAP0, TMAP0)
static double cx_kernel_e0(const scalit_ctx *c, int ntype)
{
    return (ntype == SCALIT_TA0 || ntype == SCALIT_TAAP0 || ntype == SCALIT_TMAP0) ? 0.0 : c->E0;
}

// --------------------------------------------------------------- kernels --
__global__ void cx_split_kernel(i64 n, const double *__restrict__ z, double *__restrict__ re, double *__restrict__ im)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) {
        const double2 v = reinterpret_cast<const double2 *>(z)[p];
        re[p] = v.x;
        im[p] = v.y;
    }
}

__global__ void cx_join_kernel(i64 n, const double *__restrict__ re, const double *__restrict__ im, double *__restrict__ z)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x)
        reinterpret_cast<double2 *>(z)[p] = make_double2(re[p], im[p]);
}

// Y += i sign A X on planar vectors (the imaginary part of MYHX_DX's diagonal).
__global__ void cx_absorb_kernel(i64 n, const double *__restrict__ X, double *__restrict__ Y, const double *__restrict__ A,
                                 double sign)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) {
        const double a = sign * A[p];
        const double xr = X[p], xi = X[n + p];
        Y[p] = Y[p] - a * xi;
        Y[n + p] = Y[n + p] + a * xr;
    }
}

// MYPX_DX's kernel on planar Z in place: Z / (ade + i sign A), ade = EIG0 - e0,
// clamped to +-DE inside the window for TOSBD1, alpha + (1 + beta) ade there
// for TOSBD2 (the complex form uses that expression on both sides of E0).
__global__ void cx_kernel_step(i64 n, double *__restrict__ Z, const double *__restrict__ EIG,
                               const double *__restrict__ A, double e0, double sign, int nosb, double de, double beta)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) {
        double ade = EIG[p] - e0;
        if (nosb == SCALIT_TOSBD1 && fabs(ade) <= de) ade = (ade < 0.0) ? -de : de;
        else if (nosb == SCALIT_TOSBD2 && fabs(ade) <= de) ade = -beta * de + (beta + 1.0) * ade;
        const double zr = Z[p], zi = Z[n + p];
        if (A) {
            const double ai = sign * A[p];
            const double d = ade * ade + ai * ai;
            Z[p] = (zr * ade + zi * ai) / d;
            Z[n + p] = (zi * ade - zr * ai) / d;
        } else {
            Z[p] = zr / ade;
            Z[n + p] = zi / ade;
        }
    }
}

// y = a x + b y (complex a, b) on planar vectors; overwrite: y = a x.
__global__ void cx_axpby_kernel(i64 n, double ar, double ai, const double *__restrict__ x, double br, double bi,
                                double *__restrict__ y, int overwrite)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) {
        const double xr = x[p], xi = x[n + p];
        double yr = ar * xr - ai * xi, yi = ar * xi + ai * xr;
        if (!overwrite) {
            const double vr = y[p], vi = y[n + p];
            yr += br * vr - bi * vi;
            yi += br * vi + bi * vr;
        }
        y[p] = yr;
        y[n + p] = yi;
    }
}

// y = a x for a real array a and a planar complex x.
__global__ void cx_mul_real_kernel(i64 n, const double *__restrict__ a, const double *__restrict__ x,
                                   double *__restrict__ y)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) {
        y[p] = a[p] * x[p];
        y[n + p] = a[p] * x[n + p];
    }
}

__global__ void sqrt_kernel(i64 n, const double *__restrict__ x, double *__restrict__ y)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) y[p] = sqrt(x[p]);
}

__global__ void real_div_kernel(i64 n, double *__restrict__ x, double d)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) x[p] = x[p] / d;
}

__global__ void real_mul_kernel(i64 n, double *__restrict__ x, double a)
{
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x) x[p] = a * x[p];
}

static int to_planar_n(scalit_ctx *c, i64 N, const double *Z, bool host, double *stage, double *P);
static int to_planar(scalit_ctx *c, const double *Z, bool host, double *stage, double *P);

// --------------------------------------------------------- complex window --
__global__ void gather_real_kernel(int m, const int *__restrict__ ind, const double *__restrict__ A,
                                   double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) out[i] = A[ind[i]];
}

// w = Z(ind) for planar Z (w: m real parts, then m imaginary parts)
__global__ void cx_window_gather_kernel(int m, const int *__restrict__ ind, const double *__restrict__ Z, i64 n,
                                        double *__restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) {
        w[i] = Z[ind[i]];
        w[m + i] = Z[n + ind[i]];
    }
}

// Z(ind(i)) = (HWRCX^-1 w)(i): one warp per window row (inv column-major,
// interleaved complex).
__global__ void __launch_bounds__(kT)
cx_window_solve_kernel(int m, const double2 *__restrict__ inv, const double *__restrict__ w,
                       const int *__restrict__ ind, double *__restrict__ Z, i64 n)
{
    const int row = (int)((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= m) return;
    double ar = 0.0, ai = 0.0;
    for (int j = lane; j < m; j += 32) {
        const double2 a = inv[row + (i64)j * m];
        const double wr = w[j], wi = w[m + j];
        ar += a.x * wr - a.y * wi;
        ai += a.x * wi + a.y * wr;
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (lane == 0) {
        Z[ind[row]] = ar;
        Z[n + ind[row]] = ai;
    }
}

// createWH_DXCX (src/iterate/module/osb.pij.h:63-135) for one nType: HW with
// -E0 (nTypes that use it) and +-i A(WIND) on the diagonal, inverted by
// cuSOLVER's LU (ZGETRF, then ZGETRS on the identity); kept until the nType,
// E0 or the window changes.  For TA1 the reference reads the diagonal from
// HWCX, the complex job's array, which the real job does not fill; HW is used.
static int cx_window_prepare(scalit_ctx *c, int ntype, double e0)
{
    if (c->osbw_cxinv && c->osbw_cx_ntype == ntype && c->osbw_cx_e0 == e0 && c->osbw_cx_serial == c->osbw_serial)
        return 0;
    typedef std::complex<double> cplx;
    const int m = c->osbw_len;
    cudaStream_t s = c->stream;
    CxTerms t;
    int rc = cx_terms(c, ntype, &t);
    if (rc) return rc;
    std::vector<double> hw((size_t)m * m), av((size_t)m, 0.0);
    SC_CUDA(cudaMemcpyAsync(hw.data(), c->osbw_hw, sizeof(double) * hw.size(), cudaMemcpyDeviceToHost, s));
    double *dav = nullptr;
    if (t.sign) {
        SC_CUDA(cudaMallocAsync(&dav, sizeof(double) * (size_t)m, s));
        gather_real_kernel<<<(m + kT - 1) / kT, kT, 0, s>>>(m, c->osbw_ind, t.A, dav);
        SC_CHECK_LAUNCH();
        SC_CUDA(cudaMemcpyAsync(av.data(), dav, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, s));
        cudaFreeAsync(dav, s);
    }
    SC_CUDA(cudaStreamSynchronize(s));
    std::vector<cplx> A((size_t)m * m), B((size_t)m * m, cplx(0.0, 0.0));
    for (size_t e = 0; e < A.size(); ++e) A[e] = cplx(hw[e], 0.0);
    for (int i = 0; i < m; ++i) {
        A[(size_t)i * (m + 1)] += cplx(-e0, (double)t.sign * av[(size_t)i]);
        B[(size_t)i * (m + 1)] = cplx(1.0, 0.0);
    }
    cusolverDnHandle_t sol = (cusolverDnHandle_t)c->cusolver;
    if (cusolverDnSetStream(sol, s) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnSetStream failed"); return SCALIT_ECUDA; }
    cuDoubleComplex *dA = nullptr, *dB = nullptr, *work = nullptr;
    int *ipiv = nullptr, *info = nullptr;
    auto release = [&]() {
        if (dA) cudaFreeAsync(dA, s);
        if (dB) cudaFreeAsync(dB, s);
        if (work) cudaFreeAsync(work, s);
        if (ipiv) cudaFreeAsync(ipiv, s);
        if (info) cudaFreeAsync(info, s);
    };
    if (cudaMallocAsync(&dA, sizeof(cplx) * A.size(), s) != cudaSuccess ||
        cudaMallocAsync(&dB, sizeof(cplx) * B.size(), s) != cudaSuccess ||
        cudaMallocAsync(&ipiv, sizeof(int) * (size_t)m, s) != cudaSuccess ||
        cudaMallocAsync(&info, sizeof(int) * 2, s) != cudaSuccess) {
        cudaGetLastError();
        release();
        set_error("complex window factor does not fit");
        return SCALIT_ENOMEM;
    }
    int lw = 0, hinfo[2] = {0, 0};
    do {
        if (cudaMemcpyAsync(dA, A.data(), sizeof(cplx) * A.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(dB, B.data(), sizeof(cplx) * B.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemsetAsync(info, 0, sizeof(int) * 2, s) != cudaSuccess) {
            set_error("complex window upload failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (cusolverDnZgetrf_bufferSize(sol, m, m, dA, m, &lw) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnZgetrf_bufferSize failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (cudaMallocAsync(&work, sizeof(cplx) * (size_t)std::max(lw, 1), s) != cudaSuccess) {
            cudaGetLastError();
            set_error("complex window workspace does not fit");
            rc = SCALIT_ENOMEM;
            break;
        }
        if (cusolverDnZgetrf(sol, m, m, dA, m, work, ipiv, info) != CUSOLVER_STATUS_SUCCESS ||
            cudaMemcpyAsync(hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("cusolverDnZgetrf failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (hinfo[0] != 0) {
            set_error("complex window matrix is singular (ZGETRF info=%d)", hinfo[0]);
            rc = SCALIT_EINVAL;
            break;
        }
        if (cusolverDnZgetrs(sol, CUBLAS_OP_N, m, m, dA, m, ipiv, dB, m, info + 1) != CUSOLVER_STATUS_SUCCESS ||
            cudaMemcpyAsync(hinfo + 1, info + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("cusolverDnZgetrs failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (hinfo[1] != 0) {
            set_error("complex window solve failed (ZGETRS info=%d)", hinfo[1]);
            rc = SCALIT_EINVAL;
            break;
        }
        if (!c->osbw_cxinv || c->osbw_cx_serial != c->osbw_serial) {
            if (c->osbw_cxinv) cudaFree(c->osbw_cxinv);
            if (c->osbw_cxw) cudaFree(c->osbw_cxw);
            c->osbw_cxinv = c->osbw_cxw = nullptr;
            if (cudaMalloc(&c->osbw_cxinv, sizeof(cplx) * B.size()) != cudaSuccess ||
                cudaMalloc(&c->osbw_cxw, sizeof(double) * 2 * (size_t)m) != cudaSuccess) {
                cudaGetLastError();
                set_error("complex window inverse does not fit");
                rc = SCALIT_ENOMEM;
                break;
            }
        }
        if (cudaMemcpyAsync(c->osbw_cxinv, dB, sizeof(cplx) * B.size(), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("complex window inverse copy failed");
            rc = SCALIT_ECUDA;
            break;
        }
        c->osbw_cx_ntype = ntype;
        c->osbw_cx_e0 = e0;
        c->osbw_cx_serial = c->osbw_serial;
    } while (0);
    release();
    cudaStreamSynchronize(s);
    if (rc) c->osbw_cx_serial = -1;
    return rc;
}

// -------------------------------------------------------- planar operators --
// The imaginary parts of a complex Hamiltonian's levels (sCX), added to the
// real parts' products: with H = Hr + i Hi, D = Dr + i Di (dependent level)
// and X = Xr + i Xi,
//   H X       : Yr += -Hi Xi,                       Yi += Hi Xr
//   D (H X)   : Yr += -Dr(Hi Xi) - Di(Hr Xi) - Di(Hi Xr),
//               Yi +=  Dr(Hi Xr) + Di(Hr Xr) - Di(Hi Xi)
//   outer (sNDVR, per-point A = Ar + i Ai): Yr += -Ai Xi, Yi += Ai Xr
// each a level product on the FP64 pipe with the given matrix, factors and sign.
static int hx_cx_imag_terms(const scalit_ctx *c, const double *X, double *Y, cudaStream_t s)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    const double *Xr = X, *Xi = X + N;
    double *Yr = Y, *Yi = Y + N;
    struct Term { const double *H, *D, *O, *x; double *y; double a; };
    for (int l = 0; l < L.nlev; ++l) {
        Term terms[6];
        int nt = 0;
        if (L.ndvr && l == L.nlev - 1) {
            terms[nt++] = {c->H0, c->DEP, c->OUTHi, Xi, Yr, -1.0};
            terms[nt++] = {c->H0, c->DEP, c->OUTHi, Xr, Yi, 1.0};
        } else if (!L.dep[l]) {
            terms[nt++] = {c->H0i, c->DEP, c->OUTH, Xi, Yr, -1.0};
            terms[nt++] = {c->H0i, c->DEP, c->OUTH, Xr, Yi, 1.0};
        } else {
            terms[nt++] = {c->H0i, c->DEP, c->OUTH, Xi, Yr, -1.0};
            terms[nt++] = {c->H0, c->DEPi, c->OUTH, Xi, Yr, -1.0};
            terms[nt++] = {c->H0i, c->DEPi, c->OUTH, Xr, Yr, -1.0};
            terms[nt++] = {c->H0i, c->DEP, c->OUTH, Xr, Yi, 1.0};
            terms[nt++] = {c->H0, c->DEPi, c->OUTH, Xr, Yi, 1.0};
            terms[nt++] = {c->H0i, c->DEPi, c->OUTH, Xi, Yi, -1.0};
        }
        for (int i = 0; i < nt; ++i) {
            int rc = level_apply<double>(c, l, terms[i].H, terms[i].D, terms[i].O, terms[i].x, terms[i].y,
                                         /*accumulate=*/1, nullptr, 0.0, terms[i].a, nullptr, s);
            if (rc) return rc;
        }
    }
    return 0;
}

// MYHX_DX (MYHX_CX with a complex Hamiltonian) on a planar complex vector.
static int hx_cx_planar(const scalit_ctx *c, int ntype, const double *X, double *Y, cudaStream_t s)
{
    CxTerms t;
    int rc = cx_terms(c, ntype, &t);
    if (rc) return rc;
    rc = hx_batch<double>(c, X, Y, 2, t.use_e0 ? c->E0 : 0.0, 1.0, nullptr, s);
    if (rc) return rc;
    if (c->cxh) {
        rc = hx_cx_imag_terms(c, X, Y, s);
        if (rc) return rc;
    }
    if (t.sign) {
        cx_absorb_kernel<<<cgrid(c->L.N), kT, 0, s>>>(c->L.N, X, Y, t.A, (double)t.sign);
        SC_CHECK_LAUNCH();
    }
    return 0;
}

// MYPX_DX on a planar complex vector: V^T of levels sF..1 on each half, the
// complex kernel, V of levels 1..sF (tmp: 2N).  The stages alternate between
// Y and tmp so that the last one writes Y.
static int px_cx_planar(const scalit_ctx *c, int ntype, const double *X, double *Y, double *tmp, cudaStream_t s)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
    CxTerms t;
    int rc = cx_terms(c, ntype, &t);
    if (rc) return rc;
    const bool window = c->osb_kind == SCALIT_TOSBW;
    if (window) {
        if (!(c->osbw_len > 0 && c->osbw_valid)) {
            set_error("TOSBW P*X without a window for the current preconditioner: call scalit_build_osbw again");
            return SCALIT_ESTATE;
        }
        rc = cx_window_prepare(const_cast<scalit_ctx *>(c), ntype, cx_kernel_e0(c, ntype));
        if (rc) return rc;
    }
    const int S = 2 * L.nlev;
    for (int q = 0; q < 2; ++q) {
        double *buf[2] = {Y + q * N, tmp + q * N};
        const double *in = X + q * N;
        int stage = 0;
        for (int l = L.nlev - 1; l >= 0; --l) {
            ++stage;
            double *out = buf[(S - stage) % 2];
            rc = px_rotate(c, l, 1, in, out, nullptr, s);
            if (rc) return rc;
            in = out;
        }
    }
    double *Z = (L.nlev % 2 == 0) ? Y : tmp;   // where both halves' V^T stages ended
    const int m = c->osbw_len;
    if (window) {
        cx_window_gather_kernel<<<(m + kT - 1) / kT, kT, 0, s>>>(m, c->osbw_ind, Z, N, c->osbw_cxw);
        SC_CHECK_LAUNCH();
    }
    cx_kernel_step<<<cgrid(N), kT, 0, s>>>(N, Z, c->EIG0, t.sign ? t.A : nullptr, cx_kernel_e0(c, ntype),
                                           (double)t.sign, c->osb_kind, c->osb_de, c->osb_beta);
    SC_CHECK_LAUNCH();
    if (window) {
        cx_window_solve_kernel<<<(int)(((i64)m * 32 + kT - 1) / kT), kT, 0, s>>>(
            m, reinterpret_cast<const double2 *>(c->osbw_cxinv), c->osbw_cxw, c->osbw_ind, Z, N);
        SC_CHECK_LAUNCH();
    }
    for (int q = 0; q < 2; ++q) {
        double *buf[2] = {Y + q * N, tmp + q * N};
        const double *in = Z + q * N;
        int stage = L.nlev;
        for (int l = 0; l < L.nlev; ++l) {
            ++stage;
            double *out = buf[(S - stage) % 2];
            rc = px_rotate(c, l, 0, in, out, nullptr, s);
            if (rc) return rc;
            in = out;
        }
    }
    return 0;
}

// ------------------------------------------------------------------ QMR_CX --
// QMR for the complex symmetric system (H - E0 [+-] i A) X = B with the
// complex OSB preconditioner, in the reference's order (qmrcx.f90:4-175).
// Bilinear products X^T Y (DOT_CX, vector_cx.f90:227-234) and the norms of
// the conjugated dot_product are deterministic FP64 device reductions read
// back per use; the scalar recurrence runs on the host as in the reference.
// An operator on planar device vectors: out = Op(in), scratch: 2N doubles.
typedef std::function<int(const double *in, double *out, double *scratch)> CxOp;

static int qmr_cx_core(scalit_ctx *c, i64 N, const CxOp &hxop, const CxOp &pxop, int conv, int qmrmax, double tol,
                       const double *B, double *X, int *code_out, double *res_out)
{
    typedef std::complex<double> cplx;
    const i64 N2 = 2 * N;
    cudaStream_t s = c->stream;
    double *w = nullptr, *dd = nullptr;
    const bool full_res = std::abs(conv) == 1;
    if (cudaMallocAsync(&w, sizeof(double) * (size_t)N2 * 10, s) != cudaSuccess) {
        cudaGetLastError();
        set_error("QMR_CX workspace (%lld complex points x 10) does not fit", N);
        return SCALIT_ENOMEM;
    }
    if (cudaMallocAsync(&dd, sizeof(double) * 16, s) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(w, s);
        set_error("QMR_CX scalars do not fit");
        return SCALIT_ENOMEM;
    }
    double *R = w, *UX = w + N2, *UR = w + 2 * N2, *Q = w + 3 * N2, *Sv = w + 4 * N2, *V = w + 5 * N2;
    double *Z = w + 6 * N2, *HX0 = w + 7 * N2, *T = w + 8 * N2;   // T: the preconditioner's scratch (2N)
    const int g = cgrid(N), g2 = cgrid(N2);
    int rc = 0;
    auto nrm = [&](const double *x, double *out) -> int {
        int r = dot_dev<double>(c, N2, x, x, dd, s);
        if (r) return r;
        double h;
        r = sync_read_doubles(c, dd, &h, 1);
        if (r) return r;
        *out = std::sqrt(std::fabs(h));
        return 0;
    };
    auto bil = [&](const double *x, const double *y, cplx *out) -> int {
        int r = dot_dev<double>(c, N, x, y, dd, s);
        if (!r) r = dot_dev<double>(c, N, x + N, y + N, dd + 1, s);
        if (!r) r = dot_dev<double>(c, N, x, y + N, dd + 2, s);
        if (!r) r = dot_dev<double>(c, N, x + N, y, dd + 3, s);
        if (r) return r;
        double h[4];
        r = sync_read_doubles(c, dd, h, 4);
        if (r) return r;
        *out = cplx(h[0] - h[1], h[2] + h[3]);
        return 0;
    };
    auto axpby = [&](cplx a, const double *x, cplx b, double *y, int overwrite) -> int {
        cx_axpby_kernel<<<g, kT, 0, s>>>(N, a.real(), a.imag(), x, b.real(), b.imag(), y, overwrite);
        SC_CHECK_LAUNCH();
        return 0;
    };
    auto rdiv = [&](double *x, double d) -> int {
        real_div_kernel<<<g2, kT, 0, s>>>(N2, x, d);
        SC_CHECK_LAUNCH();
        return 0;
    };
    int code = -1;
    double res = 0.0;
    do {
        double zvrat = 1.0, bnrm = 0.0, vnrm = 0.0, znrm = 0.0, gamamo = 1.0, thetamo = 0.0;
        cplx eta(-1.0, 0.0), qsdot(0.0, 0.0);
        if (conv <= 0 && cudaMemsetAsync(X, 0, sizeof(double) * (size_t)N2, s) != cudaSuccess) { set_error("memset failed"); rc = SCALIT_ECUDA; break; }
        if (cudaMemcpyAsync(R, B, sizeof(double) * (size_t)N2, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(V, B, sizeof(double) * (size_t)N2, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            set_error("QMR_CX copy failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if ((rc = nrm(B, &bnrm))) break;
        vnrm = bnrm;
        if ((rc = pxop(B, Z, T))) break;
        if ((rc = nrm(Z, &znrm))) break;
        code = 0;
        for (int i = 1; i <= qmrmax; ++i) {
            if (vnrm == 0.0 || znrm == 0.0) break;
            zvrat = zvrat * znrm / vnrm;
            if ((rc = rdiv(V, vnrm)) || (rc = rdiv(Z, znrm))) break;
            cplx vzdot;
            if ((rc = bil(V, Z, &vzdot))) break;
            if (std::abs(vzdot) == 0.0) break;
            if (i == 1) rc = axpby(cplx(1.0, 0.0), Z, cplx(0.0, 0.0), Q, 1);
            else rc = axpby(cplx(1.0, 0.0), Z, -(vnrm * vzdot) / qsdot, Q, 0);
            if (rc) break;
            if ((rc = hxop(Q, Sv, T))) break;
            real_mul_kernel<<<g2, kT, 0, s>>>(N2, Sv, zvrat);
            if (cudaGetLastError() != cudaSuccess) { set_error("QMR_CX scale launch failed"); rc = SCALIT_ECUDA; break; }
            if ((rc = bil(Q, Sv, &qsdot))) break;
            const cplx beta = qsdot / vzdot;
            if (std::abs(qsdot) == 0.0 || std::abs(beta) == 0.0) break;
            if ((rc = axpby(cplx(1.0, 0.0), Sv, -beta, V, 0))) break;
            double vnrmpo;
            if ((rc = nrm(V, &vnrmpo))) break;
            if ((rc = pxop(V, Z, T))) break;
            if ((rc = rdiv(Z, zvrat))) break;
            if ((rc = nrm(Z, &znrm))) break;
            const double theta = vnrmpo / (gamamo * std::abs(beta));
            const double gama = 1.0 / std::sqrt(1.0 + theta * theta);
            eta = -eta * vnrm * gama * gama / (beta * gamamo * gamamo);
            if (gama == 0.0) break;
            if (i == 1) {
                if ((rc = axpby(eta * zvrat, Q, cplx(0.0, 0.0), UX, 1))) break;
                if ((rc = axpby(eta, Sv, cplx(0.0, 0.0), UR, 1))) break;
            } else {
                const double tg = (thetamo * gama) * (thetamo * gama);
                if ((rc = axpby(eta * zvrat, Q, cplx(tg, 0.0), UX, 0))) break;
                if ((rc = axpby(eta, Sv, cplx(tg, 0.0), UR, 0))) break;
            }
            if ((rc = axpby(cplx(1.0, 0.0), UX, cplx(1.0, 0.0), X, 0))) break;
            if ((rc = axpby(cplx(-1.0, 0.0), UR, cplx(1.0, 0.0), R, 0))) break;
            if (full_res) {
                double xnrm, r1;
                if ((rc = hxop(X, HX0, T))) break;
                if ((rc = nrm(HX0, &xnrm))) break;
                if ((rc = axpby(cplx(-1.0, 0.0), B, cplx(1.0, 0.0), HX0, 0))) break;
                if ((rc = nrm(HX0, &r1))) break;
                res = r1 / xnrm;
            } else if (std::abs(conv) == 2) {
                double rn, uxn, xn, urn;
                if ((rc = nrm(R, &rn)) || (rc = nrm(UX, &uxn)) || (rc = nrm(X, &xn)) || (rc = nrm(UR, &urn))) break;
                res = std::max(rn / bnrm, std::max(uxn / xn, urn / rn));
            } else {
                double rn;
                if ((rc = nrm(R, &rn))) break;
                res = rn / bnrm;
            }
            if (std::fabs(res) < tol) { code = i; break; }
            code = -i;
            vnrm = vnrmpo;
            gamamo = gama;
            thetamo = theta;
        }
    } while (0);
    (void)HX0;
    cudaFreeAsync(w, s);
    cudaFreeAsync(dd, s);
    cudaStreamSynchronize(s);
    if (rc) return rc;
    *code_out = code;
    if (res_out) *res_out = res;
    return 0;
}

// QMR_CX on the context's own operators: H = MYHX_DX(ntype), P = MYPX_DX(sOSB, px_ntype).
static int qmr_cx_run(scalit_ctx *c, int conv, int qmrmax, double tol, int ntype, int px_ntype, const double *B,
                      double *X, int *code_out, double *res_out)
{
    cudaStream_t s = c->stream;
    CxOp hxop = [c, ntype, s](const double *in, double *out, double *) { return hx_cx_planar(c, ntype, in, out, s); };
    CxOp pxop = [c, px_ntype, s](const double *in, double *out, double *t) {
        return px_cx_planar(c, px_ntype, in, out, t, s);
    };
    return qmr_cx_core(c, c->L.N, hxop, pxop, conv, qmrmax, tol, B, X, code_out, res_out);
}

// ---------------------------------------------------------------------- CRP --
// osbCRP / calOSBCRP (src/iterate/module/osbw.crp.h:6-68): at each energy E
// (sOSBW%mE0 = E) NM steps of LAN_DX (lanczos/lan_dx.f90:299-325, lanHij_dx
// lanHij_dx.f90:59-97, LAN_MGS_ORTH_CX orth/gsorth_cx.f90:132-160) on the
// Hermitian operator of CRP_HXDX (:71-101): sqrt(APR) (H - E + i AP)^-1 APP
// (H - E - i AP)^-1 sqrt(APR), each inverse a QMR_CX solve.  N(E) is 4 times
// the sum of the tridiagonal's eigenvalues, i.e. 4 sum(alpha) (its trace);
// the reference's DSTEV gives the same sum to rounding.  A Lanczos breakdown
// (beta = 0) gives N(E) = 0 as LAN_DX's failure does.
static int crp_run(scalit_ctx *c, int nE, const double *energies, int nm, int qmrmax, double tol, int conv,
                   int sap, const double *X0, double *out)
{
    typedef std::complex<double> cplx;
    const i64 N = c->L.N, N2 = 2 * N;
    cudaStream_t s = c->stream;
    double *w = nullptr, *dd = nullptr;
    // five work vectors, then VJ with nm + 1 columns: step J = nm still forms
    // and normalises column nm (lanHij_dx declares VJ(N, M+1))
    const size_t ncols = (size_t)nm + 6;
    if (cudaMallocAsync(&w, sizeof(double) * (size_t)N2 * ncols, s) != cudaSuccess) {
        cudaGetLastError();
        set_error("CRP workspace (%d Lanczos vectors of %lld complex points) does not fit", (int)ncols, N);
        return SCALIT_ENOMEM;
    }
    if (cudaMallocAsync(&dd, sizeof(double) * 8, s) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(w, s);
        set_error("CRP scalars do not fit");
        return SCALIT_ENOMEM;
    }
    double *SQ = w, *W = w + N2, *Y = w + 2 * N2, *Tq = w + 3 * N2, *stage = w + 4 * N2, *VJ = w + 5 * N2;
    auto col = [&](int j) { return VJ + (i64)j * N2; };
    const int g = cgrid(N), g2 = cgrid(N2);
    const double e_saved = c->E0;
    const int pm = sap ? SCALIT_TMAP : SCALIT_TA1, pp = sap ? SCALIT_TAAP : SCALIT_TA1;
    int rc = 0;
    // the conjugated product x^H y (Fortran dot_product)
    auto hdot = [&](const double *x, const double *y, cplx *r) -> int {
        int e = dot_dev<double>(c, N, x, y, dd, s);
        if (!e) e = dot_dev<double>(c, N, x + N, y + N, dd + 1, s);
        if (!e) e = dot_dev<double>(c, N, x, y + N, dd + 2, s);
        if (!e) e = dot_dev<double>(c, N, x + N, y, dd + 3, s);
        if (e) return e;
        double h[4];
        e = sync_read_doubles(c, dd, h, 4);
        if (e) return e;
        *r = cplx(h[0] + h[1], h[2] - h[3]);
        return 0;
    };
    auto axpby = [&](cplx a, const double *x, cplx b, double *y, int overwrite) -> int {
        cx_axpby_kernel<<<g, kT, 0, s>>>(N, a.real(), a.imag(), x, b.real(), b.imag(), y, overwrite);
        SC_CHECK_LAUNCH();
        return 0;
    };
    auto mulr = [&](const double *a, const double *x, double *y) -> int {
        cx_mul_real_kernel<<<g, kT, 0, s>>>(N, a, x, y);
        SC_CHECK_LAUNCH();
        return 0;
    };
    sqrt_kernel<<<g, kT, 0, s>>>(N, c->APR, SQ);
    if (cudaGetLastError() != cudaSuccess) { set_error("CRP sqrt launch failed"); rc = SCALIT_ECUDA; }
    std::vector<double> alpha((size_t)nm), beta((size_t)nm);
    for (int e = 0; e < nE && !rc; ++e) {
        c->E0 = energies[e];
        c->gen++;
        out[e] = 0.0;
        rc = to_planar(c, X0 + (i64)e * N2, true, stage, col(0));
        if (rc) break;
        cplx t;
        if ((rc = hdot(col(0), col(0), &t))) break;
        const double tn = std::sqrt(t.real());
        if (tn == 0.0) continue;
        real_div_kernel<<<g2, kT, 0, s>>>(N2, col(0), tn);
        if (cudaGetLastError() != cudaSuccess) { set_error("CRP launch failed"); rc = SCALIT_ECUDA; break; }
        bool ok = true;
        for (int J = 1; J <= nm && !rc && ok; ++J) {
            int code = 0;
            // W = sqrt(APR) (H - E + i AP)^-1 APP (H - E - i AP)^-1 sqrt(APR) VJ(J)
            if ((rc = mulr(SQ, col(J - 1), Y))) break;
            if ((rc = qmr_cx_run(c, conv, qmrmax, tol, SCALIT_TMAP, pm, Y, Tq, &code, nullptr))) break;
            if ((rc = mulr(c->APP, Tq, Y))) break;
            if ((rc = qmr_cx_run(c, conv, qmrmax, tol, SCALIT_TAAP, pp, Y, Tq, &code, nullptr))) break;
            if ((rc = mulr(SQ, Tq, W))) break;
            if (J != 1 && (rc = axpby(cplx(-beta[(size_t)J - 2], 0.0), col(J - 2), cplx(1.0, 0.0), W, 0))) break;
            cplx a;
            if ((rc = hdot(W, col(J - 1), &a))) break;
            alpha[(size_t)J - 1] = a.real();
            for (int I = 1; I <= J; ++I) {
                cplx d;
                if ((rc = hdot(col(I - 1), W, &d))) break;
                if ((rc = axpby(-d, col(I - 1), cplx(1.0, 0.0), W, 0))) break;
            }
            if (rc) break;
            cplx nw;
            if ((rc = hdot(W, W, &nw))) break;
            const double nrm = std::sqrt(nw.real());
            beta[(size_t)J - 1] = nrm;
            if (nrm == 0.0) { ok = false; break; }
            if ((size_t)J + 5 >= ncols) {   // VJ holds columns 0..nm
                set_error("CRP Lanczos column %d outside the workspace", J);
                rc = SCALIT_ECUDA;
                break;
            }
            if (cudaMemcpyAsync(col(J), W, sizeof(double) * (size_t)N2, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
                set_error("CRP copy failed");
                rc = SCALIT_ECUDA;
                break;
            }
            real_div_kernel<<<g2, kT, 0, s>>>(N2, col(J), nrm);
            if (cudaGetLastError() != cudaSuccess) { set_error("CRP launch failed"); rc = SCALIT_ECUDA; break; }
        }
        if (rc || !ok) continue;
        double sum = 0.0;
        for (int j = 0; j < nm; ++j) sum += alpha[(size_t)j];
        out[e] = 4.0 * sum;
    }
    c->E0 = e_saved;
    c->gen++;
    cudaFreeAsync(w, s);
    cudaFreeAsync(dd, s);
    cudaStreamSynchronize(s);
    return rc;
}

// ------------------------------------------------------------------ PIST_SX --
// PIST_CONV_SX (src/iterate/libiterate/pist/pist_sx.f90:4-96) with pistH0_SX
// (pistHij_sx.f90:62-118) and MGS_ORTH_SX (orth/gsorth_sx.f90:47-72): the
// Krylov basis of the complex symmetric operator in the bilinear product,
// HMAT(I, J) = VJ_I^T H0 VJ_J, its eigenvalues (ZGEEV in the reference;
// cuSOLVER's general eigensolver here), windowed around E0 by the real part
// and tested on |lambda|^2 (getOpCX types 1 and 6, util_cx.f90:375-420).
typedef std::complex<double> cplx;

static double op_cx(int type, cplx z)
{
    return type == 1 ? z.real() : z.real() * z.real() + z.imag() * z.imag();
}

// getWindow_CX (util_cx.f90:301-325) over getWindow0 (util.f90:669-716): the
// M values closest to E0 in turn, ties to the lowest index; a short list is
// padded with its last value.
static void window_cx(double E0, int type, const std::vector<cplx> &vec, int M, std::vector<cplx> &out)
{
    const int n = (int)vec.size();
    out.assign((size_t)M, cplx(0.0, 0.0));
    if (n < M) {
        for (int i = 0; i < M; ++i) out[(size_t)i] = vec[(size_t)std::min(i, n - 1)];
        return;
    }
    std::vector<char> label((size_t)n, 1);
    for (int i = 0; i < M; ++i) {
        int best = -1;
        double bv = 0.0;
        for (int j = 0; j < n; ++j) {
            if (!label[(size_t)j]) continue;
            const double a = std::fabs(op_cx(type, vec[(size_t)j]) - E0);
            if (best < 0 || a < bv) { best = j; bv = a; }
        }
        out[(size_t)i] = vec[(size_t)best];
        label[(size_t)best] = 0;
    }
}

// Eigenvalues of the leading n x n block of HMAT (column-major, leading dimension ld).
static int geev_cx(scalit_ctx *c, int n, const std::vector<cplx> &H, int ld, std::vector<cplx> &w)
{
    cudaStream_t s = c->stream;
    cusolverDnHandle_t sol = (cusolverDnHandle_t)c->cusolver;
    if (cusolverDnSetStream(sol, s) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnSetStream failed"); return SCALIT_ECUDA; }
    std::vector<cplx> A((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) A[(size_t)i + (size_t)j * n] = H[(size_t)i + (size_t)j * ld];
    cusolverDnParams_t prm = nullptr;
    if (cusolverDnCreateParams(&prm) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnCreateParams failed"); return SCALIT_ECUDA; }
    void *dA = nullptr, *dW = nullptr, *dbuf = nullptr, *dV = nullptr;   // dV: unreferenced VL / VR
    int *dinfo = nullptr;
    std::vector<unsigned char> hbuf;
    int rc = 0;
    size_t dws = 0, hws = 0;
    do {
        if (cudaMallocAsync(&dA, sizeof(cplx) * A.size(), s) != cudaSuccess ||
            cudaMallocAsync(&dW, sizeof(cplx) * (size_t)n, s) != cudaSuccess ||
            cudaMallocAsync(&dinfo, sizeof(int), s) != cudaSuccess ||
            cudaMallocAsync(&dV, sizeof(cplx) * 2, s) != cudaSuccess) {
            cudaGetLastError();
            set_error("eigensolver buffers do not fit");
            rc = SCALIT_ENOMEM;
            break;
        }
        if (cudaMemcpyAsync(dA, A.data(), sizeof(cplx) * A.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            set_error("HMAT upload failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (cusolverDnXgeev_bufferSize(sol, prm, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_NOVECTOR, n, CUDA_C_64F,
                                       dA, n, CUDA_C_64F, dW, CUDA_C_64F, dV, 1, CUDA_C_64F, dV, 1,
                                       CUDA_C_64F, &dws, &hws) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnXgeev_bufferSize failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (cudaMallocAsync(&dbuf, std::max<size_t>(dws, 16), s) != cudaSuccess) {
            cudaGetLastError();
            set_error("eigensolver workspace does not fit");
            rc = SCALIT_ENOMEM;
            break;
        }
        hbuf.resize(std::max<size_t>(hws, 16));
        if (cudaMemsetAsync(dinfo, 0, sizeof(int), s) != cudaSuccess ||
            cusolverDnXgeev(sol, prm, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_NOVECTOR, n, CUDA_C_64F, dA, n,
                            CUDA_C_64F, dW, CUDA_C_64F, dV, 1, CUDA_C_64F, dV, 1, CUDA_C_64F, dbuf, dws,
                            hbuf.data(), hws, dinfo) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnXgeev failed");
            rc = SCALIT_ECUDA;
            break;
        }
        int info = -999;
        w.assign((size_t)n, cplx(0.0, 0.0));
        if (cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(w.data(), dW, sizeof(cplx) * (size_t)n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("eigenvalue read-back failed");
            rc = SCALIT_ECUDA;
            break;
        }
        if (info != 0) rc = 1;   // the eigensolver's own failure: PIST reports -num
    } while (0);
    if (dA) cudaFreeAsync(dA, s);
    if (dW) cudaFreeAsync(dW, s);
    if (dbuf) cudaFreeAsync(dbuf, s);
    if (dinfo) cudaFreeAsync(dinfo, s);
    if (dV) cudaFreeAsync(dV, s);
    cudaStreamSynchronize(s);
    cusolverDnDestroyParams(prm);
    return rc;
}

struct PistCxArgs {
    double e0, etol;
    int startcnt, stepcnt, stepeig, m, m_max;
    int h0_ntype, ls_ntype, ls_px_ntype, conv, qmrmax;
    double qmrtol;
    int conj;   // PIST_CONV_CX (pist/pist_cx.f90): the conjugated product throughout
};

// The linear solver of PIST: out = solve(in), *num its iteration code (<= 0 failed).
typedef std::function<int(const double *in, double *out, int *num)> CxSolve;

static int pist_cx_core(scalit_ctx *c, i64 N, const PistCxArgs &a, const double *X0, const CxOp &h0op,
                        const CxSolve &lin, std::vector<cplx> &eig, double *res_out, int *status_out)
{
    const i64 N2 = 2 * N;
    cudaStream_t s = c->stream;
    const int MM = a.m_max;
    *status_out = 0;
    eig.assign((size_t)a.m, cplx(0.0, 0.0));
    if (a.stepeig >= MM || a.startcnt > MM || a.m > MM) return 0;
    double *w = nullptr, *dd = nullptr;
    if (cudaMallocAsync(&w, sizeof(double) * (size_t)N2 * ((size_t)MM + 3), s) != cudaSuccess) {
        cudaGetLastError();
        set_error("complex PIST basis (%d vectors of %lld complex points) does not fit", MM, N);
        return SCALIT_ENOMEM;
    }
    if (cudaMallocAsync(&dd, sizeof(double) * 8, s) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(w, s);
        set_error("complex PIST scalars do not fit");
        return SCALIT_ENOMEM;
    }
    double *Wv = w, *stage = w + N2, *Xin = w + 2 * N2, *VJ = w + 3 * N2;
    auto col = [&](int j1) { return VJ + (i64)(j1 - 1) * N2; };   // 1-based
    const int g = cgrid(N);
    std::vector<cplx> H((size_t)MM * MM, cplx(0.0, 0.0));
    auto bil = [&](const double *x, const double *y, cplx *r) -> int {
        int e = dot_dev<double>(c, N, x, y, dd, s);
        if (!e) e = dot_dev<double>(c, N, x + N, y + N, dd + 1, s);
        if (!e) e = dot_dev<double>(c, N, x, y + N, dd + 2, s);
        if (!e) e = dot_dev<double>(c, N, x + N, y, dd + 3, s);
        if (e) return e;
        double h[4];
        e = sync_read_doubles(c, dd, h, 4);
        if (e) return e;
        // bilinear x^T y, or the conjugated x^H y (Fortran dot_product) for PIST_CONV_CX
        *r = a.conj ? cplx(h[0] + h[1], h[2] - h[3]) : cplx(h[0] - h[1], h[2] + h[3]);
        return 0;
    };
    auto axpby = [&](cplx al, const double *x, cplx be, double *y, int overwrite) -> int {
        cx_axpby_kernel<<<g, kT, 0, s>>>(N, al.real(), al.imag(), x, be.real(), be.imag(), y, overwrite);
        SC_CHECK_LAUNCH();
        return 0;
    };
    // the norm of MGS_ORTH_SX (principal sqrt of x^T x) or MGS_ORTH_CX (sqrt of Re x^H x)
    auto vnorm = [&](cplx d) { return a.conj ? cplx(std::sqrt(d.real()), 0.0) : std::sqrt(d); };
    // pistH0_SX / pistH0_CX: returns m_high, <= 0 from the linear solver, -J from the orthogonalisation
    auto pisth0 = [&](int m_low, int m_high, int *ret) -> int {
        *ret = 0;
        if (m_low < 1 || m_low >= m_high || m_high > MM) return 0;
        int m_start;
        if (m_low == 1) {
            m_start = 1;
            cplx xx;
            int e = bil(Xin, Xin, &xx);
            if (e) return e;
            const cplx t = vnorm(xx);
            if (t == cplx(0.0, 0.0)) return 0;
            if ((e = axpby(cplx(1.0, 0.0) / t, Xin, cplx(0.0, 0.0), col(1), 1))) return e;
        } else {
            m_start = m_low - 1;
        }
        for (int J = m_start; J <= m_high - 1; ++J) {
            int num = 0;
            int e = lin(col(J), Wv, &num);
            if (e) return e;
            if (num <= 0) { *ret = num; return 0; }
            // MGS_ORTH_SX: column J + 1 from Wv
            for (int I = 1; I <= J; ++I) {
                cplx d;
                if ((e = bil(col(I), Wv, &d))) return e;
                if ((e = axpby(-d, col(I), cplx(1.0, 0.0), Wv, 0))) return e;
            }
            cplx nw;
            if ((e = bil(Wv, Wv, &nw))) return e;
            const cplx nrm = vnorm(nw);
            if (nrm == cplx(0.0, 0.0)) { *ret = -J; return 0; }
            if ((e = axpby(cplx(1.0, 0.0) / nrm, Wv, cplx(0.0, 0.0), col(J + 1), 1))) return e;
        }
        for (int J = m_low; J <= m_high; ++J) {
            int e = h0op(col(J), Wv, nullptr);
            if (e) return e;
            for (int I = 1; I <= m_high; ++I)
                if ((e = bil(col(I), Wv, &H[(size_t)(I - 1) + (size_t)(J - 1) * MM]))) return e;
        }
        for (int J = 1; J <= m_low - 1; ++J) {
            int e = h0op(col(J), Wv, nullptr);
            if (e) return e;
            for (int I = m_low; I <= m_high; ++I)
                if ((e = bil(col(I), Wv, &H[(size_t)(I - 1) + (size_t)(J - 1) * MM]))) return e;
        }
        *ret = m_high;
        return 0;
    };
    int rc = to_planar_n(c, N, X0, true, stage, Xin);
    int status = 0;
    double res = 0.0;
    int cnt_low = 1, cnt_high = std::max(std::max(a.startcnt, a.m), a.stepeig + 1);
    std::vector<cplx> tmp, old;
    while (!rc && cnt_high <= MM) {
        int num = 0;
        if ((rc = pisth0(cnt_low, cnt_high, &num))) break;
        if (num <= 0) { status = -cnt_high; break; }
        const int n1 = cnt_high - a.stepeig;
        int g1 = geev_cx(c, n1, H, MM, tmp);
        if (g1 < 0) { rc = g1; break; }
        if (g1 > 0) { status = -n1; break; }
        window_cx(a.e0, 1, tmp, a.m, old);
        g1 = geev_cx(c, cnt_high, H, MM, tmp);
        if (g1 < 0) { rc = g1; break; }
        if (g1 > 0) { status = -cnt_high; break; }
        window_cx(a.e0, 1, tmp, a.m, eig);
        res = 0.0;
        for (int i = 0; i < a.m; ++i)
            res = std::max(res, std::fabs(op_cx(6, eig[(size_t)i]) - op_cx(6, old[(size_t)i])));
        if (res <= a.etol) { status = cnt_high; break; }
        status = -cnt_high;
        cnt_low = cnt_high + 1;
        if (cnt_low >= MM) { status = -MM; break; }
        cnt_high = std::min(cnt_high + a.stepcnt, MM);
    }
    cudaFreeAsync(w, s);
    cudaFreeAsync(dd, s);
    cudaStreamSynchronize(s);
    if (rc) return rc;
    // Reorder_CX('A', 1, ...): ascending by the real part
    std::stable_sort(eig.begin(), eig.end(), [](const cplx &x, const cplx &y) { return x.real() < y.real(); });
    *status_out = status;
    if (res_out) *res_out = res;
    return 0;
}

// PIST_CONV_SX on the context's own operators.
static int pist_cx_run(scalit_ctx *c, const PistCxArgs &a, const double *X0, std::vector<cplx> &eig, double *res_out,
                       int *status_out)
{
    cudaStream_t s = c->stream;
    CxOp h0op = [c, &a, s](const double *in, double *out, double *) { return hx_cx_planar(c, a.h0_ntype, in, out, s); };
    CxSolve lin = [c, &a](const double *in, double *out, int *num) {
        return qmr_cx_run(c, a.conv, a.qmrmax, a.qmrtol, a.ls_ntype, a.ls_px_ntype, in, out, num, nullptr);
    };
    return pist_cx_core(c, c->L.N, a, X0, h0op, lin, eig, res_out, status_out);
}

// ------------------------------------------------------------------- C ABI --
// Interleaved COMPLEX*16 in (host or device) -> planar device P (2N).
static int to_planar_n(scalit_ctx *c, i64 N, const double *Z, bool host, double *stage, double *P)
{
    const double *src = Z;
    if (host) {
        SC_CUDA(cudaMemcpyAsync(stage, Z, sizeof(double) * 2 * (size_t)N, cudaMemcpyHostToDevice, c->stream));
        src = stage;
    }
    cx_split_kernel<<<cgrid(N), kT, 0, c->stream>>>(N, src, P, P + N);
    SC_CHECK_LAUNCH();
    return 0;
}

static int to_planar(scalit_ctx *c, const double *Z, bool host, double *stage, double *P)
{
    return to_planar_n(c, c->L.N, Z, host, stage, P);
}

static int from_planar_n(scalit_ctx *c, i64 N, const double *P, bool host, double *stage, double *Z)
{
    double *dst = host ? stage : Z;
    cx_join_kernel<<<cgrid(N), kT, 0, c->stream>>>(N, P, P + N, dst);
    SC_CHECK_LAUNCH();
    if (host) SC_CUDA(cudaMemcpyAsync(Z, stage, sizeof(double) * 2 * (size_t)N, cudaMemcpyDeviceToHost, c->stream));
    return 0;
}

static int from_planar(scalit_ctx *c, const double *P, bool host, double *stage, double *Z)
{
    return from_planar_n(c, c->L.N, P, host, stage, Z);
}

// ------------------------------------------------- caller callbacks (Fortran) --
// An operator given as a caller's host callback on interleaved COMPLEX*16
// arrays: planar device in -> host -> callback -> device planar out.
struct HostCx {
    scalit_ctx *c;
    i64 N;
    double *stage;                       // device, 2N
    std::vector<double> hin, hout;
    int to_host(const double *P)
    {
        int rc = from_planar_n(c, N, P, false, nullptr, stage);
        if (rc) return rc;
        SC_CUDA(cudaMemcpyAsync(hin.data(), stage, sizeof(double) * 2 * (size_t)N, cudaMemcpyDeviceToHost, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        return 0;
    }
    int from_host(double *P) { return to_planar_n(c, N, hout.data(), true, stage, P); }
};

int qmr_cx_host(scalit_ctx *c, i64 n, scalit_fortran_op hx, scalit_fortran_op px, int conv, int qmrmax, double tol,
                const double *B, double *X, int *code, double *res)
{
    const i64 N2 = 2 * n;
    double *w = nullptr;
    SC_CUDA(cudaMallocAsync(&w, sizeof(double) * (size_t)N2 * 3, c->stream));
    HostCx h{c, n, w, std::vector<double>((size_t)N2), std::vector<double>((size_t)N2)};
    double *Bp = w + N2, *Xp = w + 2 * N2;
    const int nn = (int)n;
    auto wrap = [&](scalit_fortran_op f) {
        return CxOp([&h, f, nn](const double *in, double *out, double *) -> int {
            int rc = h.to_host(in);
            if (rc) return rc;
            f(&nn, h.hin.data(), h.hout.data());
            return h.from_host(out);
        });
    };
    int rc = to_planar_n(c, n, B, true, w, Bp);
    if (!rc && conv > 0) rc = to_planar_n(c, n, X, true, w, Xp);
    if (!rc) rc = qmr_cx_core(c, n, wrap(hx), wrap(px), conv, qmrmax, tol, Bp, Xp, code, res);
    if (!rc) rc = from_planar_n(c, n, Xp, true, w, X);
    cudaStreamSynchronize(c->stream);
    cudaFreeAsync(w, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int pist_sx_host(scalit_ctx *c, i64 n, double e0, double etol, const double *X0, int startcnt, int stepcnt,
                 int stepeig, int m, int m_max, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *eig,
                 double *res, int *status, int conj)
{
    const i64 N2 = 2 * n;
    double *w = nullptr;
    SC_CUDA(cudaMallocAsync(&w, sizeof(double) * (size_t)N2, c->stream));
    HostCx h{c, n, w, std::vector<double>((size_t)N2), std::vector<double>((size_t)N2)};
    const int nn = (int)n;
    CxOp h0op = [&h, h0x, nn](const double *in, double *out, double *) -> int {
        int rc = h.to_host(in);
        if (rc) return rc;
        h0x(&nn, h.hin.data(), h.hout.data());
        return h.from_host(out);
    };
    CxSolve lin = [&h, linsolv, nn](const double *in, double *out, int *num) -> int {
        int rc = h.to_host(in);
        if (rc) return rc;
        double r = 0.0;
        *num = linsolv(&nn, h.hin.data(), h.hout.data(), &r);
        return h.from_host(out);
    };
    PistCxArgs a{e0, etol, startcnt, stepcnt, stepeig, m, m_max, 0, 0, 0, 0, 0, 0.0, conj};
    std::vector<cplx> ev;
    int rc = pist_cx_core(c, n, a, X0, h0op, lin, ev, res, status);
    if (!rc) {
        for (int i = 0; i < m; ++i) {
            eig[2 * i] = ev[(size_t)i].real();
            eig[2 * i + 1] = ev[(size_t)i].imag();
        }
    }
    cudaFreeAsync(w, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

static int cx_apply(scalit_ctx *c, int which, int ntype, int nvec, const double *X, double *Y, bool host)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    if (!c->loaded) { set_error("complex H*X / P*X before scalit_load"); return SCALIT_ESTATE; }
    if (nvec < 0) { set_error("nvec < 0"); return SCALIT_EINVAL; }
    if (nvec == 0) return 0;
    if (!X || !Y) { set_error("null vector"); return SCALIT_EINVAL; }
    double *w = nullptr;
    if (cudaMallocAsync(&w, sizeof(double) * 2 * (size_t)N * 4, c->stream) != cudaSuccess) {
        cudaGetLastError();
        set_error("complex workspace does not fit");
        return SCALIT_ENOMEM;
    }
    double *stage = w, *P = w + 2 * N, *Qv = w + 4 * N, *T = w + 6 * N;
    int rc = 0;
    for (int v = 0; v < nvec && !rc; ++v) {
        rc = to_planar(c, X + (i64)v * 2 * N, host, stage, P);
        if (!rc) rc = which == 0 ? hx_cx_planar(c, ntype, P, Qv, c->stream) : px_cx_planar(c, ntype, P, Qv, T, c->stream);
        if (!rc) rc = from_planar(c, Qv, host, stage, Y + (i64)v * 2 * N);
    }
    cudaFreeAsync(w, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) { set_error("complex apply failed"); rc = SCALIT_ECUDA; }
    return rc;
}

}  // namespace sc

using namespace sc;

#define CX_CTX_CHECK(c)                                                           \
    do {                                                                          \
        if (!(c)) { set_error("null context"); return SCALIT_EINVAL; }            \
        if (cudaSetDevice((c)->device) != cudaSuccess) { set_error("cudaSetDevice failed"); return SCALIT_ECUDA; } \
    } while (0)

extern "C" {

int scalit_set_absorbing(scalit_ctx *c, const double *APP, const double *APR)
{
    CX_CTX_CHECK(c);
    if (!c->loaded) { set_error("scalit_set_absorbing before scalit_load"); return SCALIT_ESTATE; }
    if (!APP) { set_error("APP is required"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    for (i64 p = 0; p < N; ++p) {
        if (!std::isfinite(APP[p]) || (APR && !std::isfinite(APR[p]))) { set_error("non-finite absorbing potential"); return SCALIT_ENONFINITE; }
    }
    if (!c->AP) {
        SC_CUDA(cudaMalloc(&c->APP, sizeof(double) * (size_t)N));
        SC_CUDA(cudaMalloc(&c->APR, sizeof(double) * (size_t)N));
        SC_CUDA(cudaMalloc(&c->AP, sizeof(double) * (size_t)N));
    }
    // loadInitData (osb.io.h:18-30): JOB_RES1/2 read APP with APR = 0 and
    // AP = APP; JOB_CRP reads both and AP = APP + APR.
    std::vector<double> ap(APP, APP + N);
    if (APR) for (i64 p = 0; p < N; ++p) ap[(size_t)p] = APP[p] + APR[p];
    SC_CUDA(cudaMemcpyAsync(c->APP, APP, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, c->stream));
    if (APR) SC_CUDA(cudaMemcpyAsync(c->APR, APR, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, c->stream));
    else SC_CUDA(cudaMemsetAsync(c->APR, 0, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(c->AP, ap.data(), sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int scalit_load_cx(scalit_ctx *c, const double *H0CX, const double *RES, const double *DEPCX, const double *OUTHCX)
{
    CX_CTX_CHECK(c);
    if (!H0CX || !RES) { set_error("H0CX and RES are required"); return SCALIT_EINVAL; }
    const Layout &L = c->L;
    bool anydep = false;
    for (int l = 0; l < L.nlev; ++l) anydep = anydep || L.dep[l];
    if (anydep && !DEPCX) { set_error("a dependent level needs DEPCX"); return SCALIT_EINVAL; }
    if (L.ndvr && !OUTHCX) { set_error("sNDVR needs OUTHCX"); return SCALIT_EINVAL; }
    auto split = [](const double *z, i64 n, std::vector<double> &re, std::vector<double> &im) {
        re.resize((size_t)n);
        im.resize((size_t)n);
        for (i64 i = 0; i < n; ++i) { re[(size_t)i] = z[2 * i]; im[(size_t)i] = z[2 * i + 1]; }
    };
    std::vector<double> h0r, h0i, dr, di, orr, oi;
    split(H0CX, L.h0len, h0r, h0i);
    if (anydep) split(DEPCX, L.deplen, dr, di);
    if (L.ndvr) split(OUTHCX, L.outhlen, orr, oi);
    for (double v : h0i) if (!std::isfinite(v)) { set_error("non-finite H0CX"); return SCALIT_ENONFINITE; }
    for (double v : di) if (!std::isfinite(v)) { set_error("non-finite DEPCX"); return SCALIT_ENONFINITE; }
    for (double v : oi) if (!std::isfinite(v)) { set_error("non-finite OUTHCX"); return SCALIT_ENONFINITE; }
    c->cxh = false;
    int rc = scalit_load(c, h0r.data(), RES, anydep ? dr.data() : nullptr, L.ndvr ? orr.data() : nullptr);
    if (rc) return rc;
    auto up = [&](double **d, const std::vector<double> &h) -> int {
        if (*d) { cudaFree(*d); *d = nullptr; }
        if (h.empty()) return 0;
        SC_CUDA(cudaMalloc(d, sizeof(double) * h.size()));
        SC_CUDA(cudaMemcpyAsync(*d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, c->stream));
        return 0;
    };
    rc = up(&c->H0i, h0i);
    if (!rc) rc = up(&c->DEPi, di);
    if (!rc) rc = up(&c->OUTHi, oi);
    if (rc) return rc;
    SC_CUDA(cudaStreamSynchronize(c->stream));
    c->cxh = true;
    c->gen++;
    return 0;
}

int scalit_hx_cx(scalit_ctx *c, int ntype, int nvec, const double *X, double *Y)
{
    CX_CTX_CHECK(c);
    return cx_apply(c, 0, ntype, nvec, X, Y, true);
}

int scalit_hx_cx_device(scalit_ctx *c, int ntype, int nvec, const double *dX, double *dY)
{
    CX_CTX_CHECK(c);
    return cx_apply(c, 0, ntype, nvec, dX, dY, false);
}

int scalit_px_cx(scalit_ctx *c, int ntype, int nvec, const double *X, double *Y)
{
    CX_CTX_CHECK(c);
    return cx_apply(c, 1, ntype, nvec, X, Y, true);
}

int scalit_px_cx_device(scalit_ctx *c, int ntype, int nvec, const double *dX, double *dY)
{
    CX_CTX_CHECK(c);
    return cx_apply(c, 1, ntype, nvec, dX, dY, false);
}

int scalit_qmr_cx(scalit_ctx *c, int conv, int qmrmax, double qmrtol, int ntype, const double *B, double *X,
                  int *code, double *res)
{
    CX_CTX_CHECK(c);
    if (!c->osb_built) { set_error("QMR_CX needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    if (!B || !X || !code) { set_error("B, X and code are required"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *w = nullptr;
    SC_CUDA(cudaMallocAsync(&w, sizeof(double) * 2 * (size_t)N * 3, c->stream));
    double *stage = w, *Bp = w + 2 * N, *Xp = w + 4 * N;
    int rc = to_planar(c, B, true, stage, Bp);
    if (!rc && conv > 0) rc = to_planar(c, X, true, stage, Xp);
    if (!rc) rc = qmr_cx_run(c, conv, qmrmax, qmrtol, ntype, ntype, Bp, Xp, code, res);
    if (!rc) rc = from_planar(c, Xp, true, stage, X);
    cudaFreeAsync(w, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) { set_error("QMR_CX failed"); rc = SCALIT_ECUDA; }
    return rc;
}

int scalit_crp(scalit_ctx *c, int nenergy, const double *energies, int nm, int qmrmax, double qmrtol, int conv,
               int sap, const double *X0, double *crp)
{
    CX_CTX_CHECK(c);
    if (!c->osb_built) { set_error("CRP needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    if (!c->AP) { set_error("CRP needs the absorbing potentials: call scalit_set_absorbing"); return SCALIT_ESTATE; }
    if (nenergy < 0 || nm < 1) { set_error("CRP needs nenergy >= 0 and nm >= 1"); return SCALIT_EINVAL; }
    if (nenergy == 0) return 0;
    if (!energies || !X0 || !crp) { set_error("energies, X0 and crp are required"); return SCALIT_EINVAL; }
    return crp_run(c, nenergy, energies, nm, qmrmax, qmrtol, conv, sap, X0, crp);
}

int scalit_pist_cx(scalit_ctx *c, double e0, double etol, int ntype, int conjugate, const double *X0, int startcnt,
                   int stepcnt, int stepeig, int m, int m_max, int h0_ntype, int ls_ntype, int ls_px_ntype, int conv,
                   int qmrmax, double qmrtol, double *eig, double *res, int *status)
{
    CX_CTX_CHECK(c);
    if (!c->osb_built) { set_error("complex PIST needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    if (!X0 || !eig || !status) { set_error("X0, eig and status are required"); return SCALIT_EINVAL; }
    if (ntype > 0) {
        set_error("PIST_CONV_SX with ntype > 0 has no defined result in the reference (getSepMax_CX call)");
        return SCALIT_EUNSUP;
    }
    if (m < 1 || m_max < 2) { set_error("complex PIST needs m >= 1 and m_max >= 2"); return SCALIT_EINVAL; }
    PistCxArgs a{e0, etol, startcnt, stepcnt, stepeig, m, m_max, h0_ntype, ls_ntype, ls_px_ntype, conv, qmrmax,
                 qmrtol, conjugate ? 1 : 0};
    std::vector<cplx> ev;
    const int rc = pist_cx_run(c, a, X0, ev, res, status);
    if (rc) return rc;
    for (int i = 0; i < m; ++i) {
        eig[2 * i] = ev[(size_t)i].real();
        eig[2 * i + 1] = ev[(size_t)i].imag();
    }
    return 0;
}

}  // extern "C"
