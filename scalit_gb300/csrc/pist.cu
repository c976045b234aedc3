// PIST eigensolver on the device (PIST_CONV, src/iterate/libiterate/pist/pist.f90:7-98;
// pistH0, pistHij.f90:70-125; MGS_ORTH, src/iterate/libiterate/orth/gsorth.f90:42-72;
// window and convergence helpers, src/libutil/serial/base/util.f90:84-149,656-716).
//
// The Krylov basis VJ(N, M_MAX) and HMAT(M_MAX, M_MAX) stay in HBM in FP64.
// Modified Gram-Schmidt keeps the reference's order: one fused launch per
// previous vector applies the last projection and computes the next
// coefficient (v -= d_{i-1} u_{i-1}; d_i = v . u_i), so the vector being
// orthogonalised stays L2-resident and each basis vector is streamed once.
// HMAT columns come from one FP64 H*X and one GEMV-T per new vector; the Ritz
// values of the leading num x num block are computed by cuSOLVER's symmetric
// eigensolver (the reference calls LAPACK DSYEV at the same point); window
// selection and the convergence test run on the host over those few numbers.
#include "internal.cuh"

#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace sc {

static constexpr int kT = 256;

struct MgsState { unsigned int counter; int pad; };

__device__ __forceinline__ bool last_block(double (&acc)[1], double *partial, unsigned int *counter)
{
    __shared__ double red[kT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double a = acc[0];
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kT / 32; ++w) s += red[w];
        partial[blockIdx.x] = s;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// v -= dprev * uprev (when uprev != null); d[i] = v . u (when u != null).
__global__ void __launch_bounds__(kT)
mgs_kernel(i64 n, double *v, const double *uprev, const double *dprev, const double *u,
           double *dout, double *partial, unsigned int *counter)
{
    const double dp = uprev ? *dprev : 0.0;
    double acc[1] = {0.0};
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        double x = v[k];
        if (uprev) { x = x - dp * uprev[k]; v[k] = x; }
        const double y = u ? u[k] : x;
        acc[0] = fma(x, y, acc[0]);
    }
    if (last_block(acc, partial, counter)) {
        // every thread of the last CTA folds a fixed strided share, then a fixed tree
        __shared__ double fred[kT / 32];
        double s = 0.0;
        for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += __ldcg(&partial[b]);
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) fred[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kT / 32; ++w) t += fred[w];
            *counter = 0;
            *dout = t;
        }
    }
}

// v -= V(:, 0:m) h  (the classical Gram-Schmidt update; h staged in shared memory)
__global__ void __launch_bounds__(kT)
gemv_sub_kernel(i64 n, int m, const double *VJ, const double *h, double *v)
{
    __shared__ double hs[1024];
    for (int i0 = 0; i0 < m; i0 += 1024) {
        const int cnt = min(1024, m - i0);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) hs[i] = h[i0 + i];
        __syncthreads();
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            double a = 0.0;
            const double *col = VJ + (i64)i0 * n + k;
            for (int i = 0; i < cnt; ++i) a = fma(col[(i64)i * n], hs[i], a);
            v[k] -= a;
        }
    }
}

// h[I] = sum of the chunk partials of column I, in chunk order.
__global__ void gemvt_vec_kernel(int m, int nchunk, const double *partial, double *h)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= m) return;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += partial[(i64)I * nchunk + c];
    h[I] = s;
}

// v = v / sqrt(*nrm2) when nonzero.
__global__ void scale_inv_sqrt_kernel(i64 n, double *v, const double *nrm2)
{
    const double s = sqrt(*nrm2);
    if (s == 0.0) return;
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        v[k] = v[k] / s;
}

__global__ void copy_scaled_kernel(i64 n, const double *x, double *y, const double *nrm2)
{
    const double s = sqrt(*nrm2);
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        y[k] = x[k] / s;
}

// partial[I][chunk] = sum over the chunk of VJ(:, I) * w; then reduced in order.
static constexpr int kGemvChunk = 8192;
__global__ void __launch_bounds__(kT)
gemvt_partial_kernel(i64 n, int m, const double *VJ, const double *w, double *partial, int nchunk)
{
    const int I = blockIdx.y;
    const i64 k0 = (i64)blockIdx.x * kGemvChunk;
    const i64 k1 = min(n, k0 + kGemvChunk);
    const double *u = VJ + (i64)I * n;
    double a = 0.0;
    for (i64 k = k0 + threadIdx.x; k < k1; k += blockDim.x) a = fma(u[k], w[k], a);
    __shared__ double red[kT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w2 = 0; w2 < kT / 32; ++w2) s += red[w2];
        partial[(i64)I * nchunk + blockIdx.x] = s;
    }
    (void)m;
}

// FP32 first pass of the mixed classical Gram-Schmidt: partial[I][chunk] =
// sum over the chunk of VJf(:, I) * wf in FP32 per thread, folded in FP64.
__global__ void __launch_bounds__(kT)
gemvt_partial_f32_kernel(i64 n, const float *VJf, const float *wf, double *partial, int nchunk)
{
    const int I = blockIdx.y;
    const i64 k0 = (i64)blockIdx.x * kGemvChunk;
    const i64 k1 = min(n, k0 + kGemvChunk);
    const float *u = VJf + (i64)I * n;
    float af = 0.0f;
    for (i64 k = k0 + threadIdx.x; k < k1; k += blockDim.x) af = fmaf(u[k], wf[k], af);
    double a = (double)af;
    __shared__ double red[kT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w2 = 0; w2 < kT / 32; ++w2) s += red[w2];
        partial[(i64)I * nchunk + blockIdx.x] = s;
    }
}

// v -= VJf(:, 0:m) h with the products summed in FP32 (four interleaved
// partial sums) and the update applied to the FP64 vector.  SPLIT: h is taken
// as hi + lo, two FP32 numbers (hi = fl32(h), lo = fl32(h - hi)), and the lo
// products get their own FP32 sum, so rounding h to FP32 puts no error into
// the span of the basis (the re-orthogonalisation's update, where h is tiny).
template <bool SPLIT>
__global__ void __launch_bounds__(kT)
gemv_sub_f32_kernel(i64 n, int m, const float *VJf, const double *h, double *v)
{
    __shared__ float hs[2048];
    __shared__ float hl[SPLIT ? 2048 : 1];
    for (int i0 = 0; i0 < m; i0 += 2048) {
        const int cnt = min(2048, m - i0);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const double hd = h[i0 + i];
            const float hh = (float)hd;
            hs[i] = hh;
            if (SPLIT) hl[i] = (float)(hd - (double)hh);
        }
        __syncthreads();
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, b = 0.f;
            const float *col = VJf + (i64)i0 * n + k;
            int i = 0;
            for (; i + 3 < cnt; i += 4) {
                const float x0 = col[(i64)i * n], x1 = col[(i64)(i + 1) * n];
                const float x2 = col[(i64)(i + 2) * n], x3 = col[(i64)(i + 3) * n];
                a0 = fmaf(x0, hs[i], a0);
                a1 = fmaf(x1, hs[i + 1], a1);
                a2 = fmaf(x2, hs[i + 2], a2);
                a3 = fmaf(x3, hs[i + 3], a3);
                if (SPLIT) {
                    b = fmaf(x0, hl[i], b);
                    b = fmaf(x1, hl[i + 1], b);
                    b = fmaf(x2, hl[i + 2], b);
                    b = fmaf(x3, hl[i + 3], b);
                }
            }
            for (; i < cnt; ++i) {
                const float x0 = col[(i64)i * n];
                a0 = fmaf(x0, hs[i], a0);
                if (SPLIT) b = fmaf(x0, hl[i], b);
            }
            if (SPLIT) v[k] -= (double)((a0 + a1) + (a2 + a3)) + (double)b;
            else v[k] -= (double)((a0 + a1) + (a2 + a3));
        }
    }
}

// Vectorised forms of the two FP32 first-pass kernels, for n % 4 == 0 and
// 16-byte aligned columns: float4 loads, and the projection takes kProjVecs
// basis vectors per CTA against one register-resident chunk of wf, so the
// basis streams at full HBM rate and wf is read once per kProjVecs vectors.
static constexpr int kProjVecs = 4;
__global__ void __launch_bounds__(kT)
gemvt_partial_f32x4_kernel(i64 n, int m, const float *__restrict__ VJf, const float *__restrict__ wf,
                           double *__restrict__ partial, int nchunk)
{
    constexpr int PER = kGemvChunk / kT / 4;             // float4s per thread
    const int I0 = blockIdx.y * kProjVecs;
    const i64 k0 = (i64)blockIdx.x * kGemvChunk;
    float4 wv[PER];
    #pragma unroll
    for (int r = 0; r < PER; ++r) {
        const i64 k = k0 + 4 * ((i64)threadIdx.x + (i64)r * kT);
        wv[r] = (k < n) ? *reinterpret_cast<const float4 *>(wf + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    double a[kProjVecs];
    #pragma unroll
    for (int v = 0; v < kProjVecs; ++v) {
        float af = 0.0f;
        if (I0 + v < m) {
            const float *u = VJf + (i64)(I0 + v) * n;
            #pragma unroll
            for (int r = 0; r < PER; ++r) {
                const i64 k = k0 + 4 * ((i64)threadIdx.x + (i64)r * kT);
                if (k < n) {
                    const float4 x = *reinterpret_cast<const float4 *>(u + k);
                    af = fmaf(x.x, wv[r].x, af);
                    af = fmaf(x.y, wv[r].y, af);
                    af = fmaf(x.z, wv[r].z, af);
                    af = fmaf(x.w, wv[r].w, af);
                }
            }
        }
        a[v] = (double)af;
    }
    __shared__ double red[kT / 32][kProjVecs];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int v = 0; v < kProjVecs; ++v) {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[v] += __shfl_xor_sync(0xffffffffu, a[v], o);
    }
    if (lane == 0) {
        #pragma unroll
        for (int v = 0; v < kProjVecs; ++v) red[warp][v] = a[v];
    }
    __syncthreads();
    if (threadIdx.x < kProjVecs && I0 + (int)threadIdx.x < m) {
        double s = 0.0;
        for (int w2 = 0; w2 < kT / 32; ++w2) s += red[w2][threadIdx.x];
        partial[(i64)(I0 + threadIdx.x) * nchunk + blockIdx.x] = s;
    }
}

// v -= VJf(:, 0:m) h as gemv_sub_f32_kernel (the same four interleaved FP32
// partial sums per point and the same SPLIT form, so the same result), four
// points per thread.
template <bool SPLIT>
__global__ void __launch_bounds__(kT)
gemv_sub_f32x4_kernel(i64 n, int m, const float *__restrict__ VJf, const double *__restrict__ h,
                      double *__restrict__ v)
{
    __shared__ float hs[2048];
    __shared__ float hl[SPLIT ? 2048 : 1];
    const i64 k = 4 * (blockIdx.x * (i64)blockDim.x + threadIdx.x);
    for (int i0 = 0; i0 < m; i0 += 2048) {
        const int cnt = min(2048, m - i0);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const double hd = h[i0 + i];
            const float hh = (float)hd;
            hs[i] = hh;
            if (SPLIT) hl[i] = (float)(hd - (double)hh);
        }
        __syncthreads();
        if (k >= n) continue;
        float a[4][4];
        float bl[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        #pragma unroll
        for (int e = 0; e < 4; ++e) a[e][0] = a[e][1] = a[e][2] = a[e][3] = 0.0f;
        const float *col = VJf + (i64)i0 * n + k;
        int i = 0;
        for (; i + 3 < cnt; i += 4) {
            float4 x[4];
            #pragma unroll
            for (int j = 0; j < 4; ++j) x[j] = *reinterpret_cast<const float4 *>(col + (i64)(i + j) * n);
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float hj = hs[i + j];
                a[0][j] = fmaf(x[j].x, hj, a[0][j]);
                a[1][j] = fmaf(x[j].y, hj, a[1][j]);
                a[2][j] = fmaf(x[j].z, hj, a[2][j]);
                a[3][j] = fmaf(x[j].w, hj, a[3][j]);
                if (SPLIT) {
                    const float lj = hl[i + j];
                    bl[0] = fmaf(x[j].x, lj, bl[0]);
                    bl[1] = fmaf(x[j].y, lj, bl[1]);
                    bl[2] = fmaf(x[j].z, lj, bl[2]);
                    bl[3] = fmaf(x[j].w, lj, bl[3]);
                }
            }
        }
        for (; i < cnt; ++i) {
            const float4 x = *reinterpret_cast<const float4 *>(col + (i64)i * n);
            const float hj = hs[i];
            a[0][0] = fmaf(x.x, hj, a[0][0]);
            a[1][0] = fmaf(x.y, hj, a[1][0]);
            a[2][0] = fmaf(x.z, hj, a[2][0]);
            a[3][0] = fmaf(x.w, hj, a[3][0]);
            if (SPLIT) {
                const float lj = hl[i];
                bl[0] = fmaf(x.x, lj, bl[0]);
                bl[1] = fmaf(x.y, lj, bl[1]);
                bl[2] = fmaf(x.z, lj, bl[2]);
                bl[3] = fmaf(x.w, lj, bl[3]);
            }
        }
        double2 *vp = reinterpret_cast<double2 *>(v + k);
        double2 v0 = vp[0], v1 = vp[1];
        if (SPLIT) {
            v0.x -= (double)((a[0][0] + a[0][1]) + (a[0][2] + a[0][3])) + (double)bl[0];
            v0.y -= (double)((a[1][0] + a[1][1]) + (a[1][2] + a[1][3])) + (double)bl[1];
            v1.x -= (double)((a[2][0] + a[2][1]) + (a[2][2] + a[2][3])) + (double)bl[2];
            v1.y -= (double)((a[3][0] + a[3][1]) + (a[3][2] + a[3][3])) + (double)bl[3];
        } else {
            v0.x -= (double)((a[0][0] + a[0][1]) + (a[0][2] + a[0][3]));
            v0.y -= (double)((a[1][0] + a[1][1]) + (a[1][2] + a[1][3]));
            v1.x -= (double)((a[2][0] + a[2][1]) + (a[2][2] + a[2][3]));
            v1.y -= (double)((a[3][0] + a[3][1]) + (a[3][2] + a[3][3]));
        }
        vp[0] = v0;
        vp[1] = v1;
    }
}

__global__ void gemvt_final_kernel(int m, int nchunk, const double *partial, double *HMAT, int ld,
                                   int J)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= m) return;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += partial[(i64)I * nchunk + c];
    HMAT[I + (i64)ld * J] = s;   // HMAT(I, J)
    HMAT[J + (i64)ld * I] = s;   // HMAT(J, I)
}

// A (num x num, lda num) = symmetric matrix from the upper triangle of HMAT.
__global__ void gather_upper_kernel(int num, const double *HMAT, int ld, double *A)
{
    const i64 total = (i64)num * num;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int r = (int)(e % num), c = (int)(e / num);
        A[e] = (r <= c) ? HMAT[r + (i64)ld * c] : HMAT[c + (i64)ld * r];
    }
}

static int egrid(i64 n)
{
    i64 g = (n + kT * 4 - 1) / (kT * 4);
    if (g > 152 * 4) g = 152 * 4;
    if (g < 1) g = 1;
    return (int)g;
}

// ------------------------------------------------------- host helpers --
// getWindow0 (util.f90:669-716): M values nearest E0, chosen one at a time,
// ties resolved to the lowest index (strict '>' comparison).
static void get_window(double E0, const std::vector<double> &vec, int n, int M, double *out)
{
    if (n < M) {
        for (int i = 0; i < n; ++i) out[i] = vec[i];
        for (int i = n; i < M; ++i) out[i] = vec[n - 1];
        return;
    }
    std::vector<char> label(n, 1);
    for (int i = 0; i < M; ++i) {
        int idx = -1;
        double v0 = 0.0;
        for (int j = 0; j < n; ++j) {
            if (!label[j]) continue;
            const double a = fabs(vec[j] - E0);
            if (idx < 0 || v0 > a) { idx = j; v0 = a; }
        }
        out[i] = vec[idx];
        label[idx] = 0;
    }
}

static double diff_max(const double *a, const double *b, int n)
{
    double m = fabs(a[0] - b[0]);
    for (int i = 1; i < n; ++i) m = std::max(m, fabs(a[i] - b[i]));
    return m;
}

static double sep_max(const double *v1, int n1, const std::vector<double> &v2, int n2)
{
    double g = 0.0;
    for (int i = 0; i < n1; ++i) {
        double mm = fabs(v1[i] - v2[0]);
        for (int j = 1; j < n2; ++j) mm = std::min(mm, fabs(v1[i] - v2[j]));
        g = (i == 0) ? mm : std::max(g, mm);
    }
    return g;
}

// Ritz vectors of the M eigenvalues of HMAT(1:num, 1:num) nearest e0, ascending:
// psi = VJ(:, 1:num) y, copied to the host as M x N.
__global__ void select_columns_kernel(int num, int M, const double *Yall, const int *idx, double *Ysel)
{
    const i64 total = (i64)num * M;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int r = (int)(e % num), k = (int)(e / num);
        Ysel[e] = Yall[r + (i64)num * idx[k]];
    }
}

// partial[j][chunk] = sum over the chunk of (HPsi(:, j) - theta_j Psi(:, j))^2
__global__ void __launch_bounds__(kT)
resid_partial_kernel(i64 n, const double *Psi, const double *HPsi, const double *theta, double *partial, int nchunk)
{
    const int j = blockIdx.y;
    const i64 k0 = (i64)blockIdx.x * kGemvChunk;
    const i64 k1 = min(n, k0 + kGemvChunk);
    const double th = theta[j];
    const double *u = Psi + (i64)j * n, *hu = HPsi + (i64)j * n;
    double a = 0.0;
    for (i64 k = k0 + threadIdx.x; k < k1; k += blockDim.x) { const double r = hu[k] - th * u[k]; a = fma(r, r, a); }
    __shared__ double red[kT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w2 = 0; w2 < kT / 32; ++w2) t += red[w2];
        partial[(i64)j * nchunk + blockIdx.x] = t;
    }
}

// Ritz vectors of the window (ascending) into out_host (N x M, may be null),
// and the FP64 residual norms |H psi - theta psi|_2 of the normalised Ritz
// pairs into resid (M, may be null).
static int ritz_vectors(scalit_ctx *c, i64 N, const double *VJ, const double *HMAT, int ld, int num, double e0,
                        int M, double *A, double *EV, double *work, int lwork, int *devinfo, double *out_host,
                        double *resid = nullptr, double *eig_out = nullptr)
{
    cudaStream_t s = c->stream;
    cusolverDnHandle_t sol = (cusolverDnHandle_t)c->cusolver;
    gather_upper_kernel<<<egrid((i64)num * num), kT, 0, s>>>(num, HMAT, ld, A);
    SC_CHECK_LAUNCH();
    int lw = 0;
    if (cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, num, A, num, EV, &lw) !=
        CUSOLVER_STATUS_SUCCESS) { set_error("syevd buffer size"); return SCALIT_ECUDA; }
    double *wk = work;
    double *own = nullptr;
    if (lw > lwork) { SC_CUDA(cudaMallocAsync(&own, sizeof(double) * (size_t)lw, s)); wk = own; }
    if (cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, num, A, num, EV, wk,
                         std::max(lw, lwork), devinfo) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd (vectors) failed");
        return SCALIT_ECUDA;
    }
    std::vector<double> ev(num);
    SC_CUDA(cudaMemcpyAsync(ev.data(), EV, sizeof(double) * num, cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    // the window's indices (getWindow0's choice), then ascending by eigenvalue
    std::vector<char> label(num, 1);
    std::vector<int> idx;
    for (int i = 0; i < M && i < num; ++i) {
        int best = -1;
        double v0 = 0.0;
        for (int j = 0; j < num; ++j) {
            if (!label[j]) continue;
            const double a = fabs(ev[j] - e0);
            if (best < 0 || v0 > a) { best = j; v0 = a; }
        }
        idx.push_back(best);
        label[best] = 0;
    }
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return ev[a] < ev[b]; });
    const int Msel = (int)idx.size();
    int *didx = nullptr;
    double *Ysel = nullptr, *Psi = nullptr;
    SC_CUDA(cudaMallocAsync(&didx, sizeof(int) * Msel, s));
    SC_CUDA(cudaMallocAsync(&Ysel, sizeof(double) * (size_t)num * Msel, s));
    SC_CUDA(cudaMallocAsync(&Psi, sizeof(double) * (size_t)N * Msel, s));
    SC_CUDA(cudaMemcpyAsync(didx, idx.data(), sizeof(int) * Msel, cudaMemcpyHostToDevice, s));
    select_columns_kernel<<<egrid((i64)num * Msel), kT, 0, s>>>(num, Msel, A, didx, Ysel);
    int rc = 0;
    if (c->fp64_mode == SCALIT_FP64_TENSOR && N <= 2147483647LL) {
        // the Ritz vectors on the digit engine (a 2 N num Msel FLOP product)
        rc = tc_gemm_f64(c, (int)N, Msel, num, VJ, N, Ysel, num, Psi, N, s);
    } else {
        GemmArgs<double> g{};
        g.M = (int)N; g.N = Msel; g.K = num; g.batch = 1;
        g.Mi = N; g.s1 = 1; g.s2 = 0;
        g.A = VJ; g.a_sk = N;                 // A(p, k) = VJ[p + N k]
        g.B = Ysel; g.b_sk = 1; g.b_sn = num; // B(k, j) = Ysel[k + num j]
        g.C = Psi; g.c_sn = N;
        g.alpha = 1.0;
        rc = launch_gemm<double>(g, s);
    }
    if (eig_out)
        for (int j = 0; j < Msel; ++j) eig_out[j] = ev[idx[j]];
    if (!rc && out_host)
        SC_CUDA(cudaMemcpyAsync(out_host, Psi, sizeof(double) * (size_t)N * Msel, cudaMemcpyDeviceToHost, s));
    if (!rc && resid) {
        // H psi for all selected vectors in one batched FP64 application (HX0: no shift)
        double *HPsi = nullptr, *theta = nullptr, *part = nullptr, *rn = nullptr;
        const int nchunk = (int)((N + kGemvChunk - 1) / kGemvChunk);
        SC_CUDA(cudaMallocAsync(&HPsi, sizeof(double) * (size_t)N * Msel, s));
        SC_CUDA(cudaMallocAsync(&theta, sizeof(double) * Msel, s));
        SC_CUDA(cudaMallocAsync(&part, sizeof(double) * (size_t)nchunk * Msel, s));
        SC_CUDA(cudaMallocAsync(&rn, sizeof(double) * Msel, s));
        std::vector<double> th(Msel);
        for (int j = 0; j < Msel; ++j) th[j] = ev[idx[j]];
        SC_CUDA(cudaMemcpyAsync(theta, th.data(), sizeof(double) * Msel, cudaMemcpyHostToDevice, s));
        rc = hx_batch<double>(c, Psi, HPsi, Msel, 0.0, 1.0, nullptr, s);
        if (!rc) {
            resid_partial_kernel<<<dim3(nchunk, Msel), kT, 0, s>>>(N, Psi, HPsi, theta, part, nchunk);
            gemvt_vec_kernel<<<(Msel + 127) / 128, 128, 0, s>>>(Msel, nchunk, part, rn);
            SC_CHECK_LAUNCH();
            std::vector<double> r2(Msel);
            SC_CUDA(cudaMemcpyAsync(r2.data(), rn, sizeof(double) * Msel, cudaMemcpyDeviceToHost, s));
            SC_CUDA(cudaStreamSynchronize(s));
            for (int j = 0; j < Msel; ++j) resid[j] = std::sqrt(r2[j]);
            for (int j = Msel; j < M; ++j) resid[j] = 0.0;
        }
        cudaFreeAsync(HPsi, s); cudaFreeAsync(theta, s); cudaFreeAsync(part, s); cudaFreeAsync(rn, s);
    }
    SC_CUDA(cudaStreamSynchronize(s));
    cudaFreeAsync(didx, s); cudaFreeAsync(Ysel, s); cudaFreeAsync(Psi, s);
    if (own) cudaFreeAsync(own, s);
    return rc;
}

static double now()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int pist_core(scalit_ctx *c, i64 N, const scalit_pist_params *p, const double *dx0, PistOps &ops,
              double *eig, double *res, scalit_pist_info *info, double *vectors_host,
              const PistBasisOut *basis, double *resid, double refine_tol, int refine_max, int *refine_steps)
{
    cudaStream_t s = c->stream;
    const int M = p->m, MM = p->m_max;
    scalit_pist_info inf{};
    *res = 0.0;
    if (p->orth < 0 || p->orth > 3) { set_error("unknown orthogonalisation mode %d", p->orth); return SCALIT_EINVAL; }
    if (p->stepeig >= MM || p->startcnt > MM || M > MM || M < 1) {
        if (info) *info = inf;
        return 0;
    }
    const size_t vj_bytes = sizeof(double) * (size_t)N * MM;
    double *VJ = nullptr, *W = nullptr, *HMAT = nullptr, *A = nullptr, *EV = nullptr, *D = nullptr;
    double *partial = nullptr;
    unsigned int *counter = nullptr;
    int nchunk = (int)((N + kGemvChunk - 1) / kGemvChunk);
    if (cudaMallocAsync(&VJ, vj_bytes, s) != cudaSuccess) {
        set_error("PIST basis of %d vectors x %lld points does not fit", MM, N);
        return SCALIT_ENOMEM;
    }
    SC_CUDA(cudaMallocAsync(&W, sizeof(double) * (size_t)N, s));
    float *VJf = nullptr, *Wf = nullptr;   // FP32 copies for the mixed first pass (orth == 2)
    if (p->orth >= 2) {
        if (cudaMallocAsync(&VJf, sizeof(float) * (size_t)N * MM, s) != cudaSuccess ||
            cudaMallocAsync(&Wf, sizeof(float) * (size_t)N, s) != cudaSuccess) {
            cudaGetLastError();
            if (VJf) cudaFreeAsync(VJf, s);
            cudaFreeAsync(VJ, s); cudaFreeAsync(W, s);
            set_error("FP32 copy of the PIST basis (%d vectors x %lld points) does not fit", MM, N);
            return SCALIT_ENOMEM;
        }
    }
    auto vcolf = [&](int J1) { return VJf + (i64)(J1 - 1) * N; };
    // float4 / double2 access of every column in the mixed first pass
    const bool vec4 = VJf && N % 4 == 0 && ((reinterpret_cast<uintptr_t>(VJf) | reinterpret_cast<uintptr_t>(VJ) |
                                             reinterpret_cast<uintptr_t>(Wf)) & 15) == 0;
    SC_CUDA(cudaMallocAsync(&HMAT, sizeof(double) * (size_t)MM * MM, s));
    SC_CUDA(cudaMallocAsync(&A, sizeof(double) * (size_t)MM * MM, s));
    SC_CUDA(cudaMallocAsync(&EV, sizeof(double) * (size_t)MM, s));
    SC_CUDA(cudaMallocAsync(&D, sizeof(double) * ((size_t)MM + 8), s));
    SC_CUDA(cudaMallocAsync(&partial, sizeof(double) * std::max((size_t)nchunk * MM, (size_t)kT * 152 * 4), s));
    SC_CUDA(cudaMallocAsync(&counter, sizeof(unsigned int), s));
    SC_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
    SC_CUDA(cudaMemsetAsync(HMAT, 0, sizeof(double) * (size_t)MM * MM, s));

    cusolverDnHandle_t sol = (cusolverDnHandle_t)c->cusolver;
    int lwork = 0;
    if (cusolverDnSetStream(sol, s) != CUSOLVER_STATUS_SUCCESS ||
        cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_NOVECTOR, CUBLAS_FILL_MODE_UPPER, MM, A, MM, EV,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd_bufferSize failed");
        return SCALIT_ECUDA;
    }
    double *work = nullptr;
    int *devinfo = nullptr;
    SC_CUDA(cudaMallocAsync(&work, sizeof(double) * (size_t)std::max(lwork, 1), s));
    SC_CUDA(cudaMallocAsync(&devinfo, sizeof(int), s));

    const int gr = egrid(N);
    double *dnorm = D + MM;       // scratch scalars
    auto vcol = [&](int J1) { return VJ + (i64)(J1 - 1) * N; };   // 1-based column
    int status = 0;
    int rc = 0;

    // MGS_ORTH: orthogonalise W against columns 1..J into column J+1.
    // orth == 0: modified Gram-Schmidt in the reference's order (one pass);
    // orth == 1: classical Gram-Schmidt applied twice (GEMV-T then GEMV, x2);
    // orth == 2: the same with the first pass in FP32 against the basis' FP32
    //            copy; the second pass (the re-orthogonalisation) projects in
    //            FP64, and its update v -= V h also streams the FP32 copy: h is
    //            ~1e-7 |v| after the first pass, and the copy's rounding error
    //            (2^-24 per element, random in sign) projects onto the basis at
    //            ~1e-11, so V^T v after the update stays at FP64 round-off.
    auto mgs = [&](int J, bool *ok) -> int {
        double *v = vcol(J + 1);
        SC_CUDA(cudaMemcpyAsync(v, W, sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice, s));
        mgs_kernel<<<gr, kT, 0, s>>>(N, v, nullptr, nullptr, nullptr, dnorm, partial, counter);
        if (p->orth == 0) {
            for (int i = 1; i <= J; ++i) {
                const double *uprev = (i > 1) ? vcol(i - 1) : nullptr;
                mgs_kernel<<<gr, kT, 0, s>>>(N, v, uprev, D + (i - 2 >= 0 ? i - 2 : 0), vcol(i), D + (i - 1),
                                             partial, counter);
            }
            // last projection and the norm
            mgs_kernel<<<gr, kT, 0, s>>>(N, v, vcol(J), D + (J - 1), nullptr, dnorm + 1, partial, counter);
        } else {
            for (int pass = 0; pass < 2; ++pass) {
                if (pass == 0 && p->orth >= 2) {
                    int r2 = to_f32(v, Wf, N, s);
                    if (r2) return r2;
                    if (vec4) {
                        gemvt_partial_f32x4_kernel<<<dim3(nchunk, (J + kProjVecs - 1) / kProjVecs), kT, 0, s>>>(
                            N, J, VJf, Wf, partial, nchunk);
                    } else {
                        gemvt_partial_f32_kernel<<<dim3(nchunk, J), kT, 0, s>>>(N, VJf, Wf, partial, nchunk);
                    }
                    gemvt_vec_kernel<<<(J + 127) / 128, 128, 0, s>>>(J, nchunk, partial, D);
                    if (p->orth == 3) {
                        // the update over the FP64 basis: the FP32 copy's rounding
                        // (~6e-8 |c|) would add a component outside span(V) that
                        // the second pass cannot remove
                        gemv_sub_kernel<<<gr, kT, 0, s>>>(N, J, VJ, D, v);
                    } else if (vec4) {
                        gemv_sub_f32x4_kernel<false><<<(int)((N / 4 + kT - 1) / kT), kT, 0, s>>>(N, J, VJf, D, v);
                    } else {
                        gemv_sub_f32_kernel<false><<<gr, kT, 0, s>>>(N, J, VJf, D, v);
                    }
                    continue;
                }
                gemvt_partial_kernel<<<dim3(nchunk, J), kT, 0, s>>>(N, J, VJ, v, partial, nchunk);
                gemvt_vec_kernel<<<(J + 127) / 128, 128, 0, s>>>(J, nchunk, partial, D);
                if (p->orth >= 2 && vec4) {
                    gemv_sub_f32x4_kernel<true><<<(int)((N / 4 + kT - 1) / kT), kT, 0, s>>>(N, J, VJf, D, v);
                } else if (p->orth >= 2) {
                    gemv_sub_f32_kernel<true><<<gr, kT, 0, s>>>(N, J, VJf, D, v);
                } else {
                    gemv_sub_kernel<<<gr, kT, 0, s>>>(N, J, VJ, D, v);
                }
            }
            mgs_kernel<<<gr, kT, 0, s>>>(N, v, nullptr, nullptr, nullptr, dnorm + 1, partial, counter);
        }
        SC_CHECK_LAUNCH();
        double h[2];
        SC_CUDA(cudaMemcpyAsync(h, dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        SC_CUDA(cudaStreamSynchronize(s));
        *ok = (h[0] != 0.0) && (h[1] != 0.0);
        if (*ok) {
            scale_inv_sqrt_kernel<<<gr, kT, 0, s>>>(N, v, dnorm + 1);
            SC_CHECK_LAUNCH();
            if (VJf) {
                int r2 = to_f32(v, vcolf(J + 1), N, s);
                if (r2) return r2;
            }
        }
        return 0;
    };

    auto pisth0 = [&](int m_low, int m_high, int *ret) -> int {
        *ret = 0;
        if (m_low < 1 || m_low >= m_high || m_high > MM) return 0;
        int m_start;
        if (m_low == 1) {
            m_start = 1;
            mgs_kernel<<<gr, kT, 0, s>>>(N, const_cast<double *>(dx0), nullptr, nullptr, nullptr, dnorm,
                                         partial, counter);
            SC_CHECK_LAUNCH();
            double h;
            SC_CUDA(cudaMemcpyAsync(&h, dnorm, sizeof(double), cudaMemcpyDeviceToHost, s));
            SC_CUDA(cudaStreamSynchronize(s));
            if (h == 0.0) return 0;
            copy_scaled_kernel<<<gr, kT, 0, s>>>(N, dx0, vcol(1), dnorm);
            SC_CHECK_LAUNCH();
            if (VJf) {
                int r2 = to_f32(vcol(1), vcolf(1), N, s);
                if (r2) return r2;
            }
        } else {
            m_start = m_low - 1;
        }
        *ret = m_high;
        for (int J = m_start; J <= m_high - 1; ++J) {
            int num = 0;
            double t0 = now();
            int r = ops.linsolv(vcol(J), W, &num);
            if (r) return r;
            inf.t_qmr += now() - t0;
            inf.qmr_solves += 1;
            if (num > 0) inf.qmr_total += num;
            if (p->verbose) printf(" # of Lanczos iter.: %d . # of iter. for Linear Solver: %d\n", J, num);
            if (num <= 0) { *ret = num; return 0; }
            t0 = now();
            bool ok = false;
            r = mgs(J, &ok);
            if (r) return r;
            inf.t_orth += now() - t0;
            if (!ok) { *ret = -J; return 0; }
        }
        const double t0 = now();
        for (int J = m_low; J <= m_high; ++J) {
            int r = ops.h0x(vcol(J), W);
            if (r) return r;
            // HMAT(1:J, J) and its mirror; the rows below J come from the later columns
            gemvt_partial_kernel<<<dim3(nchunk, J), kT, 0, s>>>(N, J, VJ, W, partial, nchunk);
            gemvt_final_kernel<<<(J + 127) / 128, 128, 0, s>>>(J, nchunk, partial, HMAT, MM, J - 1);
            SC_CHECK_LAUNCH();
        }
        SC_CUDA(cudaStreamSynchronize(s));
        inf.t_hmat += now() - t0;
        return 0;
    };

    // Ritz checks.  The two DSYEV-equivalent solves of a check (leading
    // cnt_high - stepeig and cnt_high blocks of HMAT) are queued on a second
    // stream and their results read back into pinned memory; without verbose
    // output the next batch of Krylov vectors is generated while they run, and
    // the check is evaluated afterwards.  A converged check stops the solve at
    // its own cnt_high, so the eigenvalues and basis are those of the
    // sequential order; only the overlapped batch's work is spent in vain.
    std::vector<double> tmp(MM), tmp1(MM), old(M), cur(M);
    cudaStream_t s2 = c->s_out;
    double *hbuf = nullptr;
    SC_CUDA(cudaMallocHost(&hbuf, sizeof(double) * 2 * (size_t)MM + 64));
    int *hinfo = reinterpret_cast<int *>(hbuf + 2 * (size_t)MM);
    const bool overlap = !p->verbose;
    int pend_high = 0;     // cnt_high of the check queued on s2 (0: none)

    // The check's launches are issued by a worker thread: cuSOLVER's host side
    // takes ~8 ms a check at Krylov size ~500, during which the main thread
    // already queues the next batch's QMR solves (the leading high x high
    // block of HMAT that the check reads is final; later columns write rows
    // and columns beyond it).  The worker is joined before the check is
    // evaluated and before the solve returns.
    std::thread ritz_worker;
    int ritz_rc = 0;
    std::string ritz_err;
    auto ritz_launch_body = [&](int high) -> int {
        if (cusolverDnSetStream(sol, s2) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnSetStream failed"); return SCALIT_ECUDA; }
        const int nums[2] = {high - p->stepeig, high};
        for (int q = 0; q < 2; ++q) {
            const int num = nums[q];
            gather_upper_kernel<<<egrid((i64)num * num), kT, 0, s2>>>(num, HMAT, MM, A);
            SC_CHECK_LAUNCH();
            cusolverStatus_t cs = cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_NOVECTOR, CUBLAS_FILL_MODE_UPPER, num, A,
                                                   num, EV, work, lwork, devinfo);
            if (cs != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnDsyevd failed (%d)", (int)cs); return SCALIT_ECUDA; }
            SC_CUDA(cudaMemcpyAsync(hbuf + (size_t)q * MM, EV, sizeof(double) * num, cudaMemcpyDeviceToHost, s2));
            SC_CUDA(cudaMemcpyAsync(hinfo + q, devinfo, sizeof(int), cudaMemcpyDeviceToHost, s2));
        }
        inf.checks += 2;
        return 0;
    };
    auto ritz_join = [&]() -> int {
        if (ritz_worker.joinable()) ritz_worker.join();
        if (!ritz_rc) return 0;
        set_error("%s", ritz_err.c_str());     // the worker's message (errors are per thread)
        const int r = ritz_rc;
        ritz_rc = 0;
        return r;
    };
    auto ritz_launch = [&](int high) -> int {
        const int r = ritz_join();
        if (r) return r;
        pend_high = high;
        const int dev = c->device;
        ritz_worker = std::thread([&, high, dev] {
            if (cudaSetDevice(dev) != cudaSuccess) { ritz_rc = SCALIT_ECUDA; ritz_err = "cudaSetDevice failed"; return; }
            ritz_rc = ritz_launch_body(high);
            if (ritz_rc) ritz_err = scalit_last_error();
        });
        return 0;
    };
    // Evaluate the queued check (getWindow0 / getDiffMax / getSepMax on the host).
    auto ritz_settle = [&](bool *stop) -> int {
        const double t0 = now();
        {
            const int r = ritz_join();
            if (r) { pend_high = 0; return r; }
        }
        SC_CUDA(cudaStreamSynchronize(s2));
        inf.t_ritz += now() - t0;
        const int high = pend_high, num1 = high - p->stepeig;
        pend_high = 0;
        *stop = false;
        if (hinfo[0]) { status = -num1; *stop = true; return 0; }
        std::copy(hbuf, hbuf + num1, tmp1.begin());
        get_window(p->e0, tmp1, num1, M, old.data());
        if (hinfo[1]) { status = -high; *stop = true; return 0; }
        std::copy(hbuf + MM, hbuf + MM + high, tmp.begin());
        get_window(p->e0, tmp, high, M, cur.data());
        *res = (p->ntype <= 0) ? diff_max(cur.data(), old.data(), M) : sep_max(old.data(), M, tmp, high);
        if (p->verbose) printf(" Cnt1= %d  Cnt2= %d  RES= %.15e\n", high, num1, *res);
        inf.krylov = high;
        if (*res <= p->etol) { status = high; *stop = true; return 0; }
        status = -high;
        return 0;
    };

    int cnt_low = 1, cnt_high = std::max(std::max(p->startcnt, M), p->stepeig + 1);
    int built_high = 0;   // largest Krylov size whose vectors and HMAT columns are complete
    while (true) {
        int ret = 0;
        bool stop = false;
        rc = pisth0(cnt_low, cnt_high, &ret);
        if (rc) break;
        if (ret == cnt_high) built_high = cnt_high;
        if (pend_high) {
            rc = ritz_settle(&stop);
            if (rc || stop) break;
        }
        if (ret < 0) { status = -cnt_high; break; }
        if (ret == 0 && cnt_low == 1) { status = 0; set_error("PIST start vector is zero"); break; }
        rc = ritz_launch(cnt_high);
        if (rc) break;
        const bool last = cnt_high + 1 >= MM;
        if (!overlap || last) {
            rc = ritz_settle(&stop);
            if (rc || stop) break;
        }
        cnt_low = cnt_high + 1;
        if (last) { status = -MM; break; }
        cnt_high = std::min(cnt_high + p->stepcnt, MM);
    }
    {
        const int r = ritz_join();
        if (r && !rc) rc = r;
    }
    cudaStreamSynchronize(s2);
    cusolverDnSetStream(sol, s);
    if (basis && rc == 0 && status > 0) {
        const int cnt = status;
        if (basis->cnt) *basis->cnt = cnt;
        if (basis->ritz) for (int i = 0; i < cnt; ++i) basis->ritz[i] = tmp[i];
        if (basis->hmat) {
            gather_upper_kernel<<<egrid((i64)cnt * cnt), kT, 0, s>>>(cnt, HMAT, MM, A);
            if (cudaMemcpyAsync(basis->hmat, A, sizeof(double) * (size_t)cnt * cnt, cudaMemcpyDeviceToHost, s) != cudaSuccess)
                rc = SCALIT_ECUDA;
        }
        if (basis->vj && cudaMemcpyAsync(basis->vj, VJ, sizeof(double) * (size_t)N * cnt, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            rc = SCALIT_ECUDA;
        cudaStreamSynchronize(s);
        if (rc) set_error("copying the PIST basis out failed");
    }
    if (refine_steps) *refine_steps = 0;
    if (refine_tol > 0.0 && resid && rc == 0 && status > 0) {
        // Residual-based continuation: after the eigenvalue-change test, the
        // FP64 residuals |H psi - theta psi| of the window's Ritz pairs are
        // checked (Ritz vectors and one batched FP64 H*X); while one is above
        // refine_tol the basis grows by max(stepcnt, K / 20) more vectors
        // (pistH0's block step) and the check repeats, at most refine_max
        // times and up to m_max vectors.  The basis already holds the batch
        // generated while the converged check ran, so K starts there.
        const double t0 = now();
        cusolverDnSetStream(sol, s);
        int K = std::max(status, built_high), rounds = 0;
        std::vector<double> ecur((size_t)M, 0.0);
        while (true) {
            rc = ritz_vectors(c, N, VJ, HMAT, MM, K, p->e0, M, A, EV, work, lwork, devinfo, vectors_host, resid,
                              ecur.data());
            if (rc) break;
            std::copy(ecur.begin(), ecur.end(), cur.begin());
            status = K;
            inf.krylov = K;
            double rmax = 0.0;
            for (int i = 0; i < M; ++i) rmax = std::max(rmax, resid[i]);
            if (p->verbose) printf(" Cnt= %d  max FP64 residual= %.6e\n", K, rmax);
            if (rmax <= refine_tol || rounds >= refine_max || K + 1 >= MM) break;
            const int hi = std::min(MM, K + std::max(p->stepcnt, K / 20));
            int ret = 0;
            rc = pisth0(K + 1, hi, &ret);
            if (rc) break;
            if (ret != hi) break;   // the linear solver or the orthogonalisation failed: keep K
            K = hi;
            ++rounds;
        }
        if (refine_steps) *refine_steps = rounds;
        inf.t_resid += now() - t0;
    } else if ((vectors_host || resid) && rc == 0 && status > 0) {
        const double t0 = now();
        cusolverDnSetStream(sol, s);
        int r2 = ritz_vectors(c, N, VJ, HMAT, MM, status, p->e0, M, A, EV, work, lwork, devinfo, vectors_host,
                              resid);
        if (r2) rc = r2;
        inf.t_resid += now() - t0;
    }
    std::sort(cur.begin(), cur.end());
    for (int i = 0; i < M; ++i) eig[i] = cur[i];
    cudaFreeHost(hbuf);
    if (VJf) { cudaFreeAsync(VJf, s); cudaFreeAsync(Wf, s); }
    cudaFreeAsync(VJ, s); cudaFreeAsync(W, s); cudaFreeAsync(HMAT, s); cudaFreeAsync(A, s);
    cudaFreeAsync(EV, s); cudaFreeAsync(D, s); cudaFreeAsync(partial, s); cudaFreeAsync(counter, s);
    cudaFreeAsync(work, s); cudaFreeAsync(devinfo, s);
    cudaStreamSynchronize(s);
    if (info) *info = inf;
    return rc ? rc : status;
}

// pistH0 (pistHij.f90:70-125) / pistH0_MPI (pistHij_mpi.f90:83-190) on the
// caller's host arrays, as the Fortran externals pisth0_ / pisth0_mpi_ need:
// VJ(N, m_high) and HMAT(m_max, m_high), column-major, both in and out.
// Columns 1..m_low-1 of VJ (the earlier basis) are uploaded once; the new
// columns come from LinSolv and the reference's single modified Gram-Schmidt
// pass (MGS_ORTH, or MGS_ORTH_MPI with mpi = true: no initial norm test), in
// its order; column J of HMAT is V^T (H0 v_J), written with its mirror in the
// reference's order (the later column's value wins), for J = m_low..m_high.
// *num2 (may be null) receives the sum of the linear solver's codes, as
// pistH0_MPI's trailing argument.  Returns m_high, the solver's code (<= 0)
// when it failed, -J when MGS_ORTH failed at J, or 0 for bad sizes / a zero
// start vector; columns written before a failure are copied back.
int pisth0_host(scalit_ctx *c, i64 N, const double *X, int m_max, int m_low, int m_high, PistOps &ops, double *VJ,
                double *HMAT, bool mpi, int *num2, int *ret)
{
    *ret = 0;
    if (num2) *num2 = 0;
    if (m_low < 1 || m_low >= m_high || m_high > m_max || N < 1) return 0;
    cudaStream_t s = c->stream;
    const int nchunk = (int)((N + kGemvChunk - 1) / kGemvChunk);
    const int gr = egrid(N);
    double *dV = nullptr, *W = nullptr, *D = nullptr, *part = nullptr, *hcol = nullptr;
    unsigned int *counter = nullptr;
    auto fail_alloc = [&]() {
        cudaGetLastError();
        set_error("pistH0 workspace (%d vectors of %lld points) does not fit", m_high + 1, N);
        return SCALIT_ENOMEM;
    };
    int rc = 0;
    if (cudaMallocAsync(&dV, sizeof(double) * (size_t)N * m_high, s) != cudaSuccess) return fail_alloc();
    if (cudaMallocAsync(&W, sizeof(double) * (size_t)N, s) != cudaSuccess ||
        cudaMallocAsync(&D, sizeof(double) * ((size_t)m_high + 8), s) != cudaSuccess ||
        cudaMallocAsync(&part, sizeof(double) * std::max((size_t)nchunk * m_high, (size_t)kT * 152 * 4), s) != cudaSuccess ||
        cudaMallocAsync(&hcol, sizeof(double) * (size_t)m_high * (m_high - m_low + 1), s) != cudaSuccess ||
        cudaMallocAsync(&counter, sizeof(unsigned int), s) != cudaSuccess)
        rc = fail_alloc();
    auto vcol = [&](int J1) { return dV + (i64)(J1 - 1) * N; };
    double *dnorm = D + m_high;
    int m_start = 1, done_high = 0;   // columns 1..done_high of dV hold the caller's or new vectors
    if (!rc) rc = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s) == cudaSuccess ? 0 : SCALIT_ECUDA;
    if (!rc && m_low == 1) {
        double *dx = W;   // the start vector, staged in W
        if (cudaMemcpyAsync(dx, X, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            rc = SCALIT_ECUDA;
        } else {
            mgs_kernel<<<gr, kT, 0, s>>>(N, dx, nullptr, nullptr, nullptr, dnorm, part, counter);
            double h = 0.0;
            if (cudaMemcpyAsync(&h, dnorm, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                rc = SCALIT_ECUDA;
            } else if (h != 0.0) {
                copy_scaled_kernel<<<gr, kT, 0, s>>>(N, dx, vcol(1), dnorm);
                done_high = 1;
                *ret = m_high;
            }
        }
    } else if (!rc) {
        m_start = m_low - 1;
        if (cudaMemcpyAsync(dV, VJ, sizeof(double) * (size_t)N * (m_low - 1), cudaMemcpyHostToDevice, s) != cudaSuccess)
            rc = SCALIT_ECUDA;
        done_high = m_low - 1;
        *ret = m_high;
    }
    if (rc == SCALIT_ECUDA) set_error("pistH0 upload failed");
    int sum = 0;
    for (int J = m_start; !rc && *ret == m_high && J <= m_high - 1; ++J) {
        int num = 0;
        rc = ops.linsolv(vcol(J), W, &num);
        if (rc) break;
        sum += num;
        if (num <= 0) { *ret = num; break; }
        // MGS_ORTH(N, WJ, J, VJ): column J+1 = W less its projections, in order
        double *v = vcol(J + 1);
        if (cudaMemcpyAsync(v, W, sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            set_error("pistH0 copy failed");
            rc = SCALIT_ECUDA;
            break;
        }
        mgs_kernel<<<gr, kT, 0, s>>>(N, v, nullptr, nullptr, nullptr, dnorm, part, counter);
        for (int i = 1; i <= J; ++i)
            mgs_kernel<<<gr, kT, 0, s>>>(N, v, (i > 1) ? vcol(i - 1) : nullptr, D + (i > 1 ? i - 2 : 0), vcol(i),
                                         D + (i - 1), part, counter);
        mgs_kernel<<<gr, kT, 0, s>>>(N, v, vcol(J), D + (J - 1), nullptr, dnorm + 1, part, counter);
        if (cudaGetLastError() != cudaSuccess) { set_error("pistH0 launch failed"); rc = SCALIT_ECUDA; break; }
        double h[2];
        if (cudaMemcpyAsync(h, dnorm, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("pistH0 norm read failed");
            rc = SCALIT_ECUDA;
            break;
        }
        done_high = J + 1;
        if ((!mpi && h[0] == 0.0) || h[1] == 0.0) { *ret = -J; break; }
        scale_inv_sqrt_kernel<<<gr, kT, 0, s>>>(N, v, dnorm + 1);
    }
    if (num2) *num2 = sum;
    if (!rc && *ret == m_high) {
        for (int J = m_low; J <= m_high && !rc; ++J) {
            rc = ops.h0x(vcol(J), W);
            if (rc) break;
            gemvt_partial_kernel<<<dim3(nchunk, m_high), kT, 0, s>>>(N, m_high, dV, W, part, nchunk);
            gemvt_vec_kernel<<<(m_high + 127) / 128, 128, 0, s>>>(m_high, nchunk, part,
                                                                 hcol + (i64)(J - m_low) * m_high);
            if (cudaGetLastError() != cudaSuccess) { set_error("pistH0 launch failed"); rc = SCALIT_ECUDA; }
        }
        if (!rc) {
            std::vector<double> h((size_t)m_high * (m_high - m_low + 1));
            if (cudaMemcpyAsync(h.data(), hcol, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                set_error("pistH0 HMAT read failed");
                rc = SCALIT_ECUDA;
            } else {
                for (int J = m_low; J <= m_high; ++J)
                    for (int I = 1; I <= m_high; ++I) {
                        const double v = h[(size_t)(J - m_low) * m_high + (I - 1)];
                        HMAT[(I - 1) + (i64)m_max * (J - 1)] = v;
                        HMAT[(J - 1) + (i64)m_max * (I - 1)] = v;
                    }
            }
        }
    }
    // the columns this call wrote: 1 (m_low == 1) or m_low.., up to the last one formed
    const int first = (m_low == 1) ? 1 : m_low;
    if (!rc && done_high >= first &&
        cudaMemcpyAsync(VJ + (i64)(first - 1) * N, vcol(first), sizeof(double) * (size_t)N * (done_high - first + 1),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess) {
        set_error("pistH0 basis download failed");
        rc = SCALIT_ECUDA;
    }
    if (dV) cudaFreeAsync(dV, s);
    if (W) cudaFreeAsync(W, s);
    if (D) cudaFreeAsync(D, s);
    if (part) cudaFreeAsync(part, s);
    if (hcol) cudaFreeAsync(hcol, s);
    if (counter) cudaFreeAsync(counter, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) { set_error("pistH0 failed on the device"); rc = SCALIT_ECUDA; }
    return rc;
}

// Device-resident operators of the context: HX0 = MYHX(TA0), LinSolv = OSB_QMR.
struct CtxOps : PistOps {
    scalit_ctx *c;
    const scalit_pist_params *p;
    int h0x(const double *dX, double *dY) override
    {
        return hx_vec<double>(c, dX, dY, 0.0, 1.0, nullptr, c->stream);
    }
    int linsolv(const double *dB, double *dX, int *num) override
    {
        QmrResult r{};
        int rc = qmr_run(c, p->qmr_ntype, p->qmr_max, p->qmr_tol, p->precision, dB, dX, &r);
        if (rc) return rc;
        *num = r.code;
        return 0;
    }
};

int pist_ctx(scalit_ctx *c, const scalit_pist_params *p, const double *dx0, double *eig, double *res,
             scalit_pist_info *info, double *vectors_host, const PistBasisOut *basis, double *resid,
             double refine_tol, int refine_max, int *refine_steps)
{
    if (!c->osb_built) { set_error("PIST needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    CtxOps ops;
    ops.c = c;
    ops.p = p;
    return pist_core(c, c->L.N, p, dx0, ops, eig, res, info, vectors_host, basis, resid, refine_tol, refine_max,
                     refine_steps);
}

}  // namespace sc
