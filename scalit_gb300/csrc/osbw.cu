// OSBW window preconditioner (sOSB = TOSBW) for the bound-state job.
//
// initOSBW (src/iterate/module/osb.osbw.h:2-50): the window of states whose
// preconditioner eigenvalue lies within DE of E0, with DE adjusted until the
// window holds exactly sOSBW%mCnt states (adjustWinSize, :118-145); the
// window matrix HW(i, j) = <V_i | H | V_j> of the preconditioner's basis
// vectors (getVOSBH0, osb.hij.h:128-159, H = MYHX(TA0), EIG0 on the
// diagonal); HWR = HW - shift I factored by DSYTRF (createWH,
// osb.pij.h:6-45).  P*X with TOSBW (osb.px.h:191-206) solves the window
// entries with HWR and divides every other entry by EIG0 - E0.
//
// On the GPU: the window's basis vectors are Kronecker products of one VOSB
// column per level (getLevelVi, osb.vi.h:38-66), written by one kernel;
// H applied to them is one batched FP64 H*X per group of 64 vectors; HW is
// their Gram product, split over the grid points and reduced in a fixed
// order.  The reference forms H V_j again for every i < j (count^2 / 2
// H*X); here each H V_j is formed once.  HWR is factored by cuSOLVER's
// symmetric eigen-decomposition (syevd) once per window and inverted as
// Q diag(1/w) Q^T; P*X applies the inverse as a dense symmetric product (one
// warp per window row), which equals the reference's DSYTRF/DSYTRS solve to
// rounding times the condition of HWR and keeps every P*X launch
// library-free (capturable in the QMR's CUDA graphs).
#include "internal.cuh"

#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

namespace sc {

static constexpr int kT = 256;
static constexpr int kMaxAdjust = 2000;   // adjustWinSize steps before giving up
static constexpr int kBatchVecs = 64;     // window vectors per batched H*X

static int wgrid(i64 n)
{
    const i64 g = (n + kT - 1) / kT;
    return (int)std::max<i64>(1, std::min<i64>(g, 152LL * 16));
}

// ------------------------------------------------------------ window (host) --
// getOSBWSize (osb.osbw.h:62-73)
static i64 window_size(const std::vector<double> &eig, double e0, double de)
{
    i64 c = 0;
    for (double e : eig) c += (std::fabs(e - e0) <= de) ? 1 : 0;
    return c;
}

// adjustWinSize (osb.osbw.h:118-145): double DE while the window is short,
// bisect between the last two widths while it is long.  The reference loops
// without a bound; a width that holds exactly `count` states may not exist
// (tied EIG0 values), so this stops after kMaxAdjust steps.
static int adjust_width(const std::vector<double> &eig, int count, double e0, double *de)
{
    double d = *de, de1 = 0.0;
    i64 cnt0 = window_size(eig, e0, d);
    for (int it = 0; cnt0 != count; ++it) {
        if (it >= kMaxAdjust || !std::isfinite(d)) {
            set_error("no OSBW window width holds exactly %d states around E0=%.17g (tied EIG0 values)", count, e0);
            return SCALIT_EINVAL;
        }
        if (cnt0 < count) { de1 = d; d = 2.0 * d; }
        else d = 0.5 * (de1 + d);
        cnt0 = window_size(eig, e0, d);
    }
    *de = d;
    return 0;
}

// --------------------------------------------------------------- kernels --
struct WinLevels {
    int nlev;
    int n[SCALIT_FMAX];
    i64 dim[SCALIT_FMAX];
};

// getLevelVi (osb.vi.h:38-66): X[w][p] = prod_l VOSB[off[w][l] + i_l(p)],
// i_l(p) the level-l coordinate of grid point p, multiplied from level 1 up.
__global__ void osbw_basis_kernel(i64 N, WinLevels d, const double *__restrict__ VOSB, const i64 *__restrict__ off,
                                  int w0, double *__restrict__ X)
{
    const int w = blockIdx.y;
    const i64 *o = off + (i64)(w0 + w) * d.nlev;
    double *x = X + (i64)(w0 + w) * N;
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < N; p += (i64)gridDim.x * blockDim.x) {
        double acc = 1.0;
        for (int l = 0; l < d.nlev; ++l) acc = VOSB[o[l] + (p / d.dim[l]) % d.n[l]] * acc;
        x[p] = acc;
    }
}

// Split-K Gram block: P[z][I][J] = sum over the grid points of chunk z of
// X[I][p] * HX[J][p], I < mrows, J < ncols; 32 x 32 tiles, 2 x 2 per thread.
__global__ void __launch_bounds__(kT)
osbw_gram_kernel(i64 N, int mrows, int ncols, const double *__restrict__ X, const double *__restrict__ HX,
                 i64 kc, double *__restrict__ P)
{
    __shared__ double As[32][33];
    __shared__ double Bs[32][33];
    const int I0 = blockIdx.x * 32, J0 = blockIdx.y * 32, z = blockIdx.z;
    const i64 p0 = (i64)z * kc, p1 = (p0 + kc < N) ? p0 + kc : N;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double a00 = 0.0, a01 = 0.0, a10 = 0.0, a11 = 0.0;
    for (i64 k = p0; k < p1; k += 32) {
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int idx = threadIdx.x + q * kT;
            const int r = idx >> 5, cc = idx & 31;
            const i64 p = k + cc;
            As[r][cc] = (I0 + r < mrows && p < p1) ? X[(i64)(I0 + r) * N + p] : 0.0;
            Bs[r][cc] = (J0 + r < ncols && p < p1) ? HX[(i64)(J0 + r) * N + p] : 0.0;
        }
        __syncthreads();
        #pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            const double x0 = As[2 * ty][kk], x1 = As[2 * ty + 1][kk];
            const double y0 = Bs[2 * tx][kk], y1 = Bs[2 * tx + 1][kk];
            a00 = fma(x0, y0, a00);
            a01 = fma(x0, y1, a01);
            a10 = fma(x1, y0, a10);
            a11 = fma(x1, y1, a11);
        }
        __syncthreads();
    }
    const int I = I0 + 2 * ty, J = J0 + 2 * tx;
    double *Pz = P + (i64)z * mrows * ncols;
    if (I < mrows && J < ncols) Pz[(i64)I * ncols + J] = a00;
    if (I < mrows && J + 1 < ncols) Pz[(i64)I * ncols + J + 1] = a01;
    if (I + 1 < mrows && J < ncols) Pz[(i64)(I + 1) * ncols + J] = a10;
    if (I + 1 < mrows && J + 1 < ncols) Pz[(i64)(I + 1) * ncols + J + 1] = a11;
}

// HW(I, J) for the columns J = j0 .. j0+ncols-1: the chunk sums in chunk
// order for I < J, mirrored to HW(J, I); EIG0(ind(I)) on the diagonal.
__global__ void osbw_gram_reduce_kernel(int m, int mrows, int ncols, int j0, int nsplit, const double *__restrict__ P,
                                        const double *__restrict__ EIG0, const int *__restrict__ ind,
                                        double *__restrict__ HW)
{
    const i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    if (e >= (i64)mrows * ncols) return;
    const int I = (int)(e / ncols), Jl = (int)(e % ncols), J = j0 + Jl;
    if (I < J) {
        double s = 0.0;
        for (int z = 0; z < nsplit; ++z) s += P[((i64)z * mrows + I) * ncols + Jl];
        HW[I + (i64)J * m] = s;
        HW[J + (i64)I * m] = s;
    } else if (I == J) {
        HW[I + (i64)I * m] = EIG0[ind[I]];
    }
}

// A = HW - shift I (HWR, createWH osb.pij.h:20-35)
__global__ void osbw_shift_kernel(int m, const double *__restrict__ HW, double shift, double *__restrict__ A)
{
    const i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    if (e >= (i64)m * m) return;
    const int i = (int)(e % m), j = (int)(e / m);
    A[e] = HW[e] - (i == j ? shift : 0.0);
}

// A(i, j) = sum_k Q(i, k) Q(j, k) r(k), r = 1/w: the inverse from the
// eigenpairs, the same sum for (i, j) and (j, i), so A is exactly symmetric.
__global__ void osbw_inverse_kernel(int m, const double *__restrict__ Q, const double *__restrict__ r,
                                    double *__restrict__ A)
{
    const i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    if (e >= (i64)m * m) return;
    const int i = (int)(e % m), j = (int)(e / m);
    double acc = 0.0;
    for (int k = 0; k < m; ++k) acc = fma(Q[i + (i64)k * m] * Q[j + (i64)k * m], r[k], acc);
    A[e] = acc;
}

// P*X window step, in place on Z = V^T X (osb.px.h:191-206):
// 1. wy = Z(ind)
template <class T>
__global__ void osbw_gather_kernel(int m, const int *__restrict__ ind, const T *__restrict__ Z, T *__restrict__ wy,
                                   const int *gate)
{
    if (gate && *gate) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) wy[i] = Z[ind[i]];
}

// 2. Z = alpha Z / (EIG0 - E0) everywhere
template <class T>
__global__ void osbw_scale_kernel(i64 n, T *__restrict__ Z, const T *__restrict__ EIG, T e0, T alpha, const int *gate)
{
    if (gate && *gate) return;
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x)
        Z[p] = alpha * (Z[p] / (EIG[p] - e0));
}

// 3. Z(ind(i)) = alpha (HWR^-1 wy)(i): one warp per window row; the inverse
//    is stored whole, so row i is the contiguous column i.
template <class T>
__global__ void __launch_bounds__(kT)
osbw_solve_kernel(int m, const T *__restrict__ inv, const T *__restrict__ wy, const int *__restrict__ ind,
                  T *__restrict__ Z, T alpha, const int *gate)
{
    if (gate && *gate) return;
    const int row = (int)((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= m) return;
    const T *col = inv + (i64)row * m;
    T acc = T(0);
    for (int j = lane; j < m; j += 32) acc = fma(col[j], wy[j], acc);
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) Z[ind[row]] = alpha * acc;
}

// ------------------------------------------------------------------ state --
void osbw_free(scalit_ctx *c)
{
    if (c->osbw_ind) cudaFree(c->osbw_ind);
    if (c->osbw_hw) cudaFree(c->osbw_hw);
    if (c->osbw_inv) cudaFree(c->osbw_inv);
    if (c->osbw_invf) cudaFree(c->osbw_invf);
    if (c->osbw_wy) cudaFree(c->osbw_wy);
    if (c->osbw_cxinv) cudaFree(c->osbw_cxinv);
    if (c->osbw_cxw) cudaFree(c->osbw_cxw);
    c->osbw_cxinv = c->osbw_cxw = nullptr;
    c->osbw_cx_serial = -1;
    c->osbw_ind = nullptr;
    c->osbw_hw = c->osbw_inv = nullptr;
    c->osbw_invf = nullptr;
    c->osbw_wy = nullptr;
    c->osbw_len = 0;
    c->osbw_valid = false;
}

void osbw_invalidate(scalit_ctx *c)
{
    c->osbw_valid = false;
}

// HW from the window's basis vectors: X (count x N) resident, H applied in
// groups of kBatchVecs, each group's Gram block reduced into HW.
static int form_hw(scalit_ctx *c, int m, const int *d_ind, const std::vector<i64> &offs, double *HW, cudaStream_t s)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    const int nb = std::min(m, kBatchVecs);
    double *X = nullptr, *HX = nullptr, *P = nullptr;
    i64 *d_off = nullptr;
    auto release = [&]() {
        if (X) cudaFreeAsync(X, s);
        if (HX) cudaFreeAsync(HX, s);
        if (P) cudaFreeAsync(P, s);
        if (d_off) cudaFreeAsync(d_off, s);
    };
    if (cudaMallocAsync(&X, sizeof(double) * (size_t)m * N, s) != cudaSuccess ||
        cudaMallocAsync(&HX, sizeof(double) * (size_t)nb * N, s) != cudaSuccess) {
        cudaGetLastError();
        release();
        set_error("OSBW: the %d window basis vectors (%lld points each) do not fit", m, N);
        return SCALIT_ENOMEM;
    }
    const int tiles_max = ((m + 31) / 32) * ((nb + 31) / 32);
    int nsplit = std::max(1, (152 * 4 + tiles_max - 1) / tiles_max);
    nsplit = (int)std::min<i64>(nsplit, std::max<i64>(1, N / 1024));
    const i64 kc = (N + nsplit - 1) / nsplit;
    if (cudaMallocAsync(&P, sizeof(double) * (size_t)nsplit * m * nb, s) != cudaSuccess ||
        cudaMallocAsync(&d_off, sizeof(i64) * offs.size(), s) != cudaSuccess) {
        cudaGetLastError();
        release();
        set_error("OSBW: Gram workspace does not fit");
        return SCALIT_ENOMEM;
    }
    int rc = 0;
    if (cudaMemcpyAsync(d_off, offs.data(), sizeof(i64) * offs.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) {
        set_error("OSBW: offsets upload failed");
        rc = SCALIT_ECUDA;
    }
    WinLevels wl{};
    wl.nlev = L.nlev;
    for (int l = 0; l < L.nlev; ++l) { wl.n[l] = L.n[l]; wl.dim[l] = L.dim[l]; }
    for (int w0 = 0; w0 < m && !rc; w0 += 65535) {
        const int cnt = std::min(65535, m - w0);
        osbw_basis_kernel<<<dim3(std::min(wgrid(N), 1024), cnt), kT, 0, s>>>(N, wl, c->VOSB, d_off, w0, X);
        if (cudaGetLastError() != cudaSuccess) { set_error("OSBW basis launch failed"); rc = SCALIT_ECUDA; }
    }
    for (int j0 = 0; j0 < m && !rc; j0 += nb) {
        const int ncols = std::min(nb, m - j0);
        const int mrows = std::min(m, j0 + ncols);     // HW(I, J) is formed for I <= J only
        rc = hx_batch<double>(c, X + (i64)j0 * N, HX, ncols, 0.0, 1.0, nullptr, s);
        if (rc) break;
        osbw_gram_kernel<<<dim3((mrows + 31) / 32, (ncols + 31) / 32, nsplit), kT, 0, s>>>(N, mrows, ncols, X, HX,
                                                                                          kc, P);
        const i64 ne = (i64)mrows * ncols;
        osbw_gram_reduce_kernel<<<(int)((ne + kT - 1) / kT), kT, 0, s>>>(m, mrows, ncols, j0, nsplit, P, c->EIG0,
                                                                         d_ind, HW);
        if (cudaGetLastError() != cudaSuccess) { set_error("OSBW Gram launch failed"); rc = SCALIT_ECUDA; }
    }
    release();
    return rc;
}

// HWR = HW - shift I -> its inverse (both triangles, FP64 and FP32) from the
// symmetric eigen-decomposition HWR = Q diag(w) Q^T (cuSOLVER syevd):
// HWR^-1 = Q diag(1/w) Q^T.  An exactly zero eigenvalue is the singular case
// DSYTRF reports with info > 0 (createWH fails).
static int invert_hwr(scalit_ctx *c, int m, double shift, cudaStream_t s)
{
    const i64 mm = (i64)m * m;
    const int g = (int)((mm + kT - 1) / kT);
    cusolverDnHandle_t sol = (cusolverDnHandle_t)c->cusolver;
    if (cusolverDnSetStream(sol, s) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnSetStream failed"); return SCALIT_ECUDA; }
    double *Q = nullptr, *w = nullptr, *work = nullptr;
    int *info = nullptr;
    auto release = [&]() {
        if (Q) cudaFreeAsync(Q, s);
        if (w) cudaFreeAsync(w, s);
        if (work) cudaFreeAsync(work, s);
        if (info) cudaFreeAsync(info, s);
    };
    if (cudaMallocAsync(&Q, sizeof(double) * (size_t)mm, s) != cudaSuccess ||
        cudaMallocAsync(&w, sizeof(double) * (size_t)m, s) != cudaSuccess ||
        cudaMallocAsync(&info, sizeof(int), s) != cudaSuccess) {
        cudaGetLastError();
        release();
        set_error("OSBW: factor workspace does not fit");
        return SCALIT_ENOMEM;
    }
    osbw_shift_kernel<<<g, kT, 0, s>>>(m, c->osbw_hw, shift, Q);
    int rc = 0;
    if (cudaGetLastError() != cudaSuccess) { set_error("OSBW shift launch failed"); rc = SCALIT_ECUDA; }
    int lw = 0;
    if (!rc && cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, m, Q, m, w, &lw) !=
                   CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd_bufferSize failed");
        rc = SCALIT_ECUDA;
    }
    if (!rc && cudaMallocAsync(&work, sizeof(double) * (size_t)std::max(lw, 1), s) != cudaSuccess) {
        cudaGetLastError();
        set_error("OSBW: eigensolver workspace does not fit");
        rc = SCALIT_ENOMEM;
    }
    if (!rc && cudaMemsetAsync(info, 0, sizeof(int), s) != cudaSuccess) { set_error("memset failed"); rc = SCALIT_ECUDA; }
    if (!rc && cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, m, Q, m, w, work, std::max(lw, 1),
                                info) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd failed");
        rc = SCALIT_ECUDA;
    }
    int hinfo = 0;
    std::vector<double> hw((size_t)m);
    if (!rc && (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaMemcpyAsync(hw.data(), w, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)) {
        set_error("OSBW eigenvalue read-back failed");
        rc = SCALIT_ECUDA;
    }
    if (!rc && hinfo != 0) {
        set_error("OSBW window matrix eigen-decomposition failed (syevd info=%d)", hinfo);
        rc = SCALIT_EINVAL;
    }
    if (!rc) {
        for (int k = 0; k < m; ++k) {
            if (hw[(size_t)k] == 0.0 || !std::isfinite(hw[(size_t)k])) {
                set_error("OSBW window matrix HW - E0 is singular (eigenvalue %d is %g)", k + 1, hw[(size_t)k]);
                rc = SCALIT_EINVAL;
                break;
            }
        }
    }
    if (!rc) {
        for (int k = 0; k < m; ++k) hw[(size_t)k] = 1.0 / hw[(size_t)k];
        if (cudaMemcpyAsync(w, hw.data(), sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("OSBW reciprocal upload failed");
            rc = SCALIT_ECUDA;
        }
    }
    if (!rc) {
        osbw_inverse_kernel<<<g, kT, 0, s>>>(m, Q, w, c->osbw_inv);
        if (cudaGetLastError() != cudaSuccess) { set_error("OSBW inverse launch failed"); rc = SCALIT_ECUDA; }
    }
    release();
    if (rc) return rc;
    return to_f32(c->osbw_inv, c->osbw_invf, mm, s);
}

int osbw_make(scalit_ctx *c, double e0, int count, double *de, int npc, const double *hw_host, int *hwlen)
{
    const Layout &L = c->L;
    if (!c->osb_built) { set_error("OSBW needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    if (!de) { set_error("de is required"); return SCALIT_EINVAL; }
    if (count < 1 || (i64)count > L.N) { set_error("OSBW window size %d outside 1..N", count); return SCALIT_EINVAL; }
    if (!(*de > 0.0) || !std::isfinite(*de) || !std::isfinite(e0)) {
        set_error("OSBW needs a finite E0 and a starting width DE > 0");
        return SCALIT_EINVAL;
    }
    if (npc != SCALIT_TA0 && npc != SCALIT_TA1) { set_error("npc must be TA0 or TA1"); return SCALIT_EINVAL; }
    cudaStream_t s = c->stream;
    std::vector<double> eig((size_t)L.N);
    SC_CUDA(cudaMemcpyAsync(eig.data(), c->EIG0, sizeof(double) * (size_t)L.N, cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    double d = *de;
    int rc = adjust_width(eig, count, e0, &d);
    if (rc) return rc;
    // getOSBWIndex (osb.osbw.h:76-92) and getLevelIndex (osb.vi.h:11-27):
    // the window's points in ascending order and, per level, the VOSB offset
    // of the column its basis vector takes (block = the slower levels'
    // coordinates, column = the level's own coordinate).
    std::vector<int> ind;
    ind.reserve((size_t)count);
    for (i64 p = 0; p < L.N && (int)ind.size() < count; ++p)
        if (std::fabs(eig[(size_t)p] - e0) <= d) ind.push_back((int)p);
    const int m = (int)ind.size();
    std::vector<i64> offs((size_t)m * L.nlev);
    for (int w = 0; w < m; ++w) {
        for (int l = 0; l < L.nlev; ++l) {
            const i64 clen = L.dim[l] * L.n[l];
            const i64 bk = ind[(size_t)w] / clen;
            const i64 col = (ind[(size_t)w] - bk * clen) / L.dim[l];
            offs[(size_t)w * L.nlev + l] = L.vs[l] + bk * L.n[l] * L.n[l] + col * L.n[l];
        }
    }
    osbw_free(c);
    const i64 mm = (i64)m * m;
    if (cudaMalloc(&c->osbw_ind, sizeof(int) * (size_t)m) != cudaSuccess ||
        cudaMalloc(&c->osbw_hw, sizeof(double) * (size_t)mm) != cudaSuccess ||
        cudaMalloc(&c->osbw_inv, sizeof(double) * (size_t)mm) != cudaSuccess ||
        cudaMalloc(&c->osbw_invf, sizeof(float) * (size_t)mm) != cudaSuccess ||
        cudaMalloc(&c->osbw_wy, sizeof(double) * (size_t)m) != cudaSuccess) {
        cudaGetLastError();
        osbw_free(c);
        set_error("OSBW window of %d states does not fit", m);
        return SCALIT_ENOMEM;
    }
    SC_CUDA(cudaMemcpyAsync(c->osbw_ind, ind.data(), sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, s));
    if (hw_host) {
        SC_CUDA(cudaMemcpyAsync(c->osbw_hw, hw_host, sizeof(double) * (size_t)mm, cudaMemcpyHostToDevice, s));
    } else {
        rc = form_hw(c, m, c->osbw_ind, offs, c->osbw_hw, s);
        if (rc) { osbw_free(c); return rc; }
    }
    rc = invert_hwr(c, m, npc == SCALIT_TA1 ? e0 : 0.0, s);
    if (rc) { osbw_free(c); return rc; }
    SC_CUDA(cudaStreamSynchronize(s));
    c->osbw_len = m;
    c->osbw_valid = true;
    c->osbw_serial++;
    c->osbw_e0 = e0;
    c->osbw_de = d;
    c->osb_kind = SCALIT_TOSBW;
    c->gen++;
    *de = d;
    if (hwlen) *hwlen = m;
    return 0;
}

template <class T>
int osbw_window_apply(const scalit_ctx *c, T *Z, const T *EIG, double e0, T alpha, const int *gate, cudaStream_t s)
{
    const int m = c->osbw_len;
    const T *inv;
    if constexpr (std::is_same<T, double>::value) inv = c->osbw_inv;
    else inv = c->osbw_invf;
    T *wy = static_cast<T *>(c->osbw_wy);
    osbw_gather_kernel<T><<<(m + kT - 1) / kT, kT, 0, s>>>(m, c->osbw_ind, Z, wy, gate);
    osbw_scale_kernel<T><<<wgrid(c->L.N), kT, 0, s>>>(c->L.N, Z, EIG, T(e0), alpha, gate);
    osbw_solve_kernel<T><<<(int)(((i64)m * 32 + kT - 1) / kT), kT, 0, s>>>(m, inv, wy, c->osbw_ind, Z, alpha, gate);
    SC_CHECK_LAUNCH();
    return 0;
}

template int osbw_window_apply<double>(const scalit_ctx *, double *, const double *, double, double, const int *, cudaStream_t);
template int osbw_window_apply<float>(const scalit_ctx *, float *, const float *, double, float, const int *, cudaStream_t);

}  // namespace sc
