// Device-resident preconditioned QMR (QMR, src/iterate/libiterate/qmr/qmr.f90:5-175;
// breakdown codes of QMR_MPI, src/iterate/libiterate_mpi/qmr/qmr_mpi.f90:4-263).
//
// Every scalar of the recurrence lives in a device struct; the vector steps
// are fused elementwise + reduction kernels whose last CTA to finish folds the
// per-CTA partial sums in a fixed order (deterministic) and then advances the
// scalar recurrence.  Every kernel first reads the struct's `done` flag and
// returns when it is set, so the host can queue several iterations ahead and
// only reads the flag back between batches.  The H*X and P*X launches take
// the same flag as their gate.  FP32 mode keeps the vectors in FP32 and
// accumulates every reduction in FP64.
#include "internal.cuh"

#include <cmath>
#include <vector>

namespace sc {

static constexpr int kRedThreads = 256;
static constexpr int kRedMaxBlocks = 152 * 4;
// per right-hand side: room for 4 partial sums of every CTA of a reduction
static constexpr i64 kPartStride = 4 * kRedMaxBlocks;

struct QmrState {
    double BNRM, ZNRM, VNRM, VNRMPO, ZVRAT, QSDOT, VZDOT, BETA, ETA;
    double GAMAMO, GAMA, THETAMO, THETA, RES, XNRM;
    double fq;        // Q = Z - fq * Q
    double cq, cs, g; // UX = cq Q + g UX ; UR = cs S + g UR
    double inv_zvrat;
    double tol;
    int i, code, done, qmrmax, ntype, iters, breakdown;
    unsigned int counter;
};

// Sum of the per-CTA partials (NV values per CTA), by every thread of the last
// CTA: a fixed strided split, then a fixed warp/CTA tree -- the same order on
// every run.  The result is valid in thread 0.
template <int NV>
__device__ __forceinline__ void fold(const double *partial, int nblk, double (&out)[NV])
{
    __shared__ double fred[NV][kRedThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double a[NV];
    #pragma unroll
    for (int v = 0; v < NV; ++v) a[v] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        #pragma unroll
        for (int v = 0; v < NV; ++v) a[v] += __ldcg(&partial[NV * b + v]);
    #pragma unroll
    for (int v = 0; v < NV; ++v) {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[v] += __shfl_xor_sync(0xffffffffu, a[v], o);
        if (lane == 0) fred[v][warp] = a[v];
    }
    __syncthreads();
    #pragma unroll
    for (int v = 0; v < NV; ++v) {
        double s = 0.0;
        for (int w = 0; w < kRedThreads / 32; ++w) s += fred[v][w];
        out[v] = s;
    }
}

template <int NV>
__device__ __forceinline__ bool block_reduce_store(double (&acc)[NV], double *partial,
                                                   unsigned int *counter)
{
    __shared__ double red[NV][kRedThreads / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int v = 0; v < NV; ++v) {
        double a = acc[v];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[v][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        #pragma unroll
        for (int v = 0; v < NV; ++v) {
            double a = 0.0;
            for (int w = 0; w < kRedThreads / 32; ++w) a += red[v][w];
            partial[NV * blockIdx.x + v] = a;
        }
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// FP32 steps on float4 groups (n % 4 == 0): the group's products are summed
// in FP32 and the group sum is added to the FP64 accumulator -- one
// conversion and one FP64 add per four points instead of per point (on this
// part FP64 arithmetic and conversions share the slow FP64 pipe).
template <class T> __device__ __forceinline__ bool use_vec4(i64 n)
{
    return sizeof(T) == 4 && (n & 3) == 0;
}
__device__ __forceinline__ float dot4(const float4 a, const float4 b)
{
    return fmaf(a.x, b.x, a.y * b.y) + fmaf(a.z, b.z, a.w * b.w);
}
#define SC_GRID_LOOP4(k4, n4) \
    for (i64 k4 = blockIdx.x * (i64)blockDim.x + threadIdx.x; k4 < (n4); k4 += (i64)gridDim.x * blockDim.x)

// ----------------------------------------------------------------- steps --
// step A: V /= VNRM, Z /= ZNRM, VZDOT = V.Z
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_a(i64 n, i64 ld, T *V, T *Z, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; V += y * ld; Z += y * ld; st += y; partial += y * kPartStride; }
    if (st->done) return;
    const double vn = st->VNRM, zn = st->ZNRM;
    if (vn == 0.0 || zn == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) { st->code = -1; st->breakdown = 1; st->done = 1; }
        return;
    }
    const T tv = T(vn), tz = T(zn);
    double acc[1] = {0.0};
    if (use_vec4<T>(n)) {
        float4 *V4 = reinterpret_cast<float4 *>(V), *Z4 = reinterpret_cast<float4 *>(Z);
        const float fv = (float)tv, fz = (float)tz;
        SC_GRID_LOOP4(k4, n >> 2) {
            float4 v = V4[k4], z = Z4[k4];
            v.x /= fv; v.y /= fv; v.z /= fv; v.w /= fv;
            z.x /= fz; z.y /= fz; z.z /= fz; z.w /= fz;
            V4[k4] = v; Z4[k4] = z;
            acc[0] += (double)dot4(v, z);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T v = V[k] / tv, z = Z[k] / tz;
            V[k] = v; Z[k] = z;
            acc[0] += (double)v * (double)z;
        }
    }
    if (block_reduce_store<1>(acc, partial, &st->counter)) {
        double d[1];
        fold<1>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->ZVRAT = st->ZVRAT * st->ZNRM / st->VNRM;
        st->VZDOT = d[0];
        st->inv_zvrat = 1.0 / st->ZVRAT;
        if (st->VZDOT == 0.0) { st->code = -2; st->breakdown = 1; st->done = 1; return; }
        st->fq = (st->i == 1) ? 0.0 : st->VNRM * st->VZDOT / st->QSDOT;
    }
}

// step B: Q = Z (i == 1) or Z - fq Q
template <class T>
__global__ void qmr_step_b(i64 n, i64 ld, const T *Z, T *Q, const QmrState *st)
{
    { const int y = blockIdx.y; Z += y * ld; Q += y * ld; st += y; }
    if (st->done) return;
    const bool first = (st->i == 1);
    const T f = T(st->fq);
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        Q[k] = first ? Z[k] : Z[k] - f * Q[k];
}

// step C: S = ZVRAT S, QSDOT = Q.S, BETA = QSDOT / VZDOT
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_c(i64 n, i64 ld, const T *Q, T *S, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; Q += y * ld; S += y * ld; st += y; partial += y * kPartStride; }
    if (st->done) return;
    const T zv = T(st->ZVRAT);
    double acc[1] = {0.0};
    if (use_vec4<T>(n)) {
        const float4 *Q4 = reinterpret_cast<const float4 *>(Q);
        float4 *S4 = reinterpret_cast<float4 *>(S);
        const float f = (float)zv;
        SC_GRID_LOOP4(k4, n >> 2) {
            float4 sv = S4[k4];
            sv.x *= f; sv.y *= f; sv.z *= f; sv.w *= f;
            S4[k4] = sv;
            acc[0] += (double)dot4(Q4[k4], sv);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T sv = zv * S[k];
            S[k] = sv;
            acc[0] += (double)Q[k] * (double)sv;
        }
    }
    if (block_reduce_store<1>(acc, partial, &st->counter)) {
        double d[1];
        fold<1>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->QSDOT = d[0];
        st->BETA = st->QSDOT / st->VZDOT;
        if (st->QSDOT == 0.0 || st->BETA == 0.0) { st->code = -3; st->breakdown = 1; st->done = 1; }
    }
}

// step D: V = S - BETA V, VNRMPO = |V|
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_d(i64 n, i64 ld, const T *S, T *V, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; S += y * ld; V += y * ld; st += y; partial += y * kPartStride; }
    if (st->done) return;
    const T beta = T(st->BETA);
    double acc[1] = {0.0};
    if (use_vec4<T>(n)) {
        const float4 *S4 = reinterpret_cast<const float4 *>(S);
        float4 *V4 = reinterpret_cast<float4 *>(V);
        const float b = (float)beta;
        SC_GRID_LOOP4(k4, n >> 2) {
            const float4 sv = S4[k4];
            float4 v = V4[k4];
            v.x = sv.x - b * v.x; v.y = sv.y - b * v.y; v.z = sv.z - b * v.z; v.w = sv.w - b * v.w;
            V4[k4] = v;
            acc[0] += (double)dot4(v, v);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T v = S[k] - beta * V[k];
            V[k] = v;
            acc[0] += (double)v * (double)v;
        }
    }
    if (block_reduce_store<1>(acc, partial, &st->counter)) {
        double d[1];
        fold<1>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->VNRMPO = sqrt(d[0]);
    }
}

// step E: Z = Z / ZVRAT, ZNRM = |Z|, then THETA, GAMA, ETA and the X/R update coefficients
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_e(i64 n, i64 ld, T *Z, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; Z += y * ld; st += y; partial += y * kPartStride; }
    if (st->done) return;
    const T zv = T(st->ZVRAT);
    double acc[1] = {0.0};
    if (use_vec4<T>(n)) {
        float4 *Z4 = reinterpret_cast<float4 *>(Z);
        const float f = (float)zv;
        SC_GRID_LOOP4(k4, n >> 2) {
            float4 z = Z4[k4];
            z.x /= f; z.y /= f; z.z /= f; z.w /= f;
            Z4[k4] = z;
            acc[0] += (double)dot4(z, z);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T z = Z[k] / zv;
            Z[k] = z;
            acc[0] += (double)z * (double)z;
        }
    }
    if (block_reduce_store<1>(acc, partial, &st->counter)) {
        double d[1];
        fold<1>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->ZNRM = sqrt(d[0]);
        st->THETA = st->VNRMPO / (st->GAMAMO * fabs(st->BETA));
        st->GAMA = 1.0 / sqrt(1.0 + st->THETA * st->THETA);
        st->ETA = -st->ETA * st->VNRM * st->GAMA * st->GAMA / (st->BETA * st->GAMAMO * st->GAMAMO);
        if (st->GAMA == 0.0) { st->code = -4; st->breakdown = 1; st->done = 1; return; }
        st->cq = st->ETA * st->ZVRAT;
        st->cs = st->ETA;
        const double tg = st->THETAMO * st->GAMA;
        st->g = (st->i == 1) ? 0.0 : tg * tg;
    }
}

__device__ void qmr_advance(QmrState *st)
{
    if (fabs(st->RES) < st->tol) {
        st->code = st->i;
        st->iters = st->i;
        st->done = 1;
        return;
    }
    st->code = -st->i;
    st->iters = st->i;
    st->VNRM = st->VNRMPO;
    st->GAMAMO = st->GAMA;
    st->THETAMO = st->THETA;
    st->i = st->i + 1;
    if (st->i > st->qmrmax) st->done = 1;
}

// step F: UX, UR, X, R updates; for ntype != +-1 also the convergence test.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_f(i64 n, i64 ld, const T *Q, const T *S, T *UX, T *UR, T *X, T *R, QmrState *st, double *partial)
{
    {
        const int y = blockIdx.y;
        Q += y * ld; S += y * ld; UX += y * ld; UR += y * ld; X += y * ld; R += y * ld;
        st += y; partial += y * kPartStride;
    }
    if (st->done) return;
    const bool first = (st->i == 1);
    const T cq = T(st->cq), cs = T(st->cs), g = T(st->g);
    const int conv = abs(st->ntype);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    if (use_vec4<T>(n)) {
        const float4 *Q4 = reinterpret_cast<const float4 *>(Q), *S4 = reinterpret_cast<const float4 *>(S);
        float4 *UX4 = reinterpret_cast<float4 *>(UX), *UR4 = reinterpret_cast<float4 *>(UR);
        float4 *X4 = reinterpret_cast<float4 *>(X), *R4 = reinterpret_cast<float4 *>(R);
        const float fq = (float)cq, fs = (float)cs, fg = (float)g;
        SC_GRID_LOOP4(k4, n >> 2) {
            const float4 q = Q4[k4], sv = S4[k4];
            float4 ux, ur;
            if (first) {
                ux = make_float4(fq * q.x, fq * q.y, fq * q.z, fq * q.w);
                ur = make_float4(fs * sv.x, fs * sv.y, fs * sv.z, fs * sv.w);
            } else {
                const float4 u0 = UX4[k4], u1 = UR4[k4];
                ux = make_float4(fq * q.x + fg * u0.x, fq * q.y + fg * u0.y, fq * q.z + fg * u0.z, fq * q.w + fg * u0.w);
                ur = make_float4(fs * sv.x + fg * u1.x, fs * sv.y + fg * u1.y, fs * sv.z + fg * u1.z,
                                 fs * sv.w + fg * u1.w);
            }
            UX4[k4] = ux; UR4[k4] = ur;
            float4 x = X4[k4], r = R4[k4];
            x.x += ux.x; x.y += ux.y; x.z += ux.z; x.w += ux.w;
            r.x -= ur.x; r.y -= ur.y; r.z -= ur.z; r.w -= ur.w;
            X4[k4] = x; R4[k4] = r;
            if (conv != 1) {
                acc[0] += (double)dot4(r, r);
                acc[1] += (double)dot4(ux, ux);
                acc[2] += (double)dot4(x, x);
                acc[3] += (double)dot4(ur, ur);
            }
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T ux = first ? cq * Q[k] : cq * Q[k] + g * UX[k];
            const T ur = first ? cs * S[k] : cs * S[k] + g * UR[k];
            UX[k] = ux; UR[k] = ur;
            const T x = X[k] + ux, r = R[k] - ur;
            X[k] = x; R[k] = r;
            acc[0] += (double)r * (double)r;
            acc[1] += (double)ux * (double)ux;
            acc[2] += (double)x * (double)x;
            acc[3] += (double)ur * (double)ur;
        }
    }
    if (conv == 1) return;  // the |HX-B|/|HX| test follows in step G
    if (block_reduce_store<4>(acc, partial, &st->counter)) {
        double d[4];
        fold<4>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        if (conv == 2) {
            const double r1 = sqrt(d[0]) / st->BNRM;
            const double r2 = sqrt(d[1] / d[2]);
            const double r3 = sqrt(d[3] / d[0]);
            st->RES = fmax(fmax(r1, r2), r3);
        } else {
            st->RES = sqrt(d[0]) / st->BNRM;
        }
        qmr_advance(st);
    }
}

// step G: XNRM = |HX0|, RES = |HX0 - B| / XNRM (HX0 = H X), then advance.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_step_g(i64 n, i64 ld, const T *HX0, const T *B, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; HX0 += y * ld; B += y * ld; st += y; partial += y * kPartStride; }
    if (st->done) return;
    double acc[2] = {0.0, 0.0};
    if (use_vec4<T>(n)) {
        const float4 *H4 = reinterpret_cast<const float4 *>(HX0), *B4 = reinterpret_cast<const float4 *>(B);
        SC_GRID_LOOP4(k4, n >> 2) {
            const float4 h = H4[k4], b = B4[k4];
            const float4 d = make_float4(h.x - b.x, h.y - b.y, h.z - b.z, h.w - b.w);
            acc[0] += (double)dot4(h, h);
            acc[1] += (double)dot4(d, d);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            const T h = HX0[k];
            const T d = h - B[k];
            acc[0] += (double)h * (double)h;
            acc[1] += (double)d * (double)d;
        }
    }
    if (block_reduce_store<2>(acc, partial, &st->counter)) {
        double d[2];
        fold<2>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->XNRM = sqrt(d[0]);
        st->RES = sqrt(d[1]) / st->XNRM;
        qmr_advance(st);
    }
}

// initial norms: BNRM = VNRM = |B|, ZNRM = |Z|
template <class T>
__global__ void __launch_bounds__(kRedThreads)
qmr_init_norms(i64 n, i64 ld, const T *B, const T *Z, QmrState *st, double *partial)
{
    { const int y = blockIdx.y; B += y * ld; Z += y * ld; st += y; partial += y * kPartStride; }
    double acc[2] = {0.0, 0.0};
    if (use_vec4<T>(n)) {
        const float4 *B4 = reinterpret_cast<const float4 *>(B), *Z4 = reinterpret_cast<const float4 *>(Z);
        SC_GRID_LOOP4(k4, n >> 2) {
            const float4 b = B4[k4], z = Z4[k4];
            acc[0] += (double)dot4(b, b);
            acc[1] += (double)dot4(z, z);
        }
    } else {
        for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
            acc[0] += (double)B[k] * (double)B[k];
            acc[1] += (double)Z[k] * (double)Z[k];
        }
    }
    if (block_reduce_store<2>(acc, partial, &st->counter)) {
        double d[2];
        fold<2>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        st->counter = 0;
        st->BNRM = sqrt(d[0]);
        st->VNRM = st->BNRM;
        st->ZNRM = sqrt(d[1]);
        if (st->qmrmax < 1) st->done = 1;
    }
}

// Stop flags of the right-hand sides' states, for per-vector gating of the operators.
const int *qmr_done_flag(const QmrState *st) { return &st->done; }
int qmr_state_stride() { return (int)(sizeof(QmrState) / sizeof(int)); }

// all = 1 when every right-hand side's recurrence has stopped
__global__ void qmr_all_done(const QmrState *st, int nrhs, int *all)
{
    int d = 1;
    for (int v = threadIdx.x; v < nrhs; v += blockDim.x) d &= st[v].done ? 1 : 0;
    d = __all_sync(0xffffffffu, d);
    if (threadIdx.x == 0) *all = d;
}

template <class T>
__global__ void copy_kernel(i64 n, const T *a, T *b, T *c)
{
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x) {
        const T v = a[k];
        b[k] = v;
        if (c) c[k] = v;
    }
}

__global__ void f64_to_f32_kernel(i64 n, const double *x, float *y)
{
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        y[k] = (float)x[k];
}

__global__ void f32_to_f64_kernel(i64 n, const float *x, double *y)
{
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        y[k] = (double)x[k];
}

static int red_grid(i64 n)
{
    i64 g = (n + kRedThreads * 4 - 1) / (kRedThreads * 4);
    if (g > kRedMaxBlocks) g = kRedMaxBlocks;
    if (g < 1) g = 1;
    return (int)g;
}

static int ew_grid(i64 n)
{
    i64 g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return (int)g;
}

int to_f32(const double *x, float *y, i64 n, cudaStream_t s)
{
    if (n <= 0) return 0;
    f64_to_f32_kernel<<<ew_grid(n), 256, 0, s>>>(n, x, y);
    SC_CHECK_LAUNCH();
    return 0;
}

int to_f64(const float *x, double *y, i64 n, cudaStream_t s)
{
    if (n <= 0) return 0;
    f32_to_f64_kernel<<<ew_grid(n), 256, 0, s>>>(n, x, y);
    SC_CHECK_LAUNCH();
    return 0;
}

__global__ void axpy_kernel(i64 n, double a, const double *x, double *y)
{
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        y[k] = y[k] + a * x[k];
}

__global__ void scal_kernel(i64 n, double a, double *x)
{
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        x[k] = a * x[k];
}

int axpy_dev(i64 n, double a, const double *x, double *y, cudaStream_t s)
{
    if (n <= 0) return 0;
    axpy_kernel<<<ew_grid(n), 256, 0, s>>>(n, a, x, y);
    SC_CHECK_LAUNCH();
    return 0;
}

int scal_dev(i64 n, double a, double *x, cudaStream_t s)
{
    if (n <= 0) return 0;
    scal_kernel<<<ew_grid(n), 256, 0, s>>>(n, a, x);
    SC_CHECK_LAUNCH();
    return 0;
}

// Plain deterministic dot for the API (NORM_MPI / DOTPROD_MPI drop-ins).
template <class T>
__global__ void __launch_bounds__(kRedThreads)
dot_kernel(i64 n, const T *x, const T *y, double *partial, unsigned int *counter, double *out)
{
    double acc[1] = {0.0};
    for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < n; k += (i64)gridDim.x * blockDim.x)
        acc[0] += (double)x[k] * (double)y[k];
    if (block_reduce_store<1>(acc, partial, counter)) {
        double d[1];
        fold<1>(partial, gridDim.x, d);
        if (threadIdx.x != 0) return;
        *counter = 0;
        *out = d[0];
    }
}

template <class T>
int dot_dev(scalit_ctx *c, i64 n, const T *x, const T *y, double *out, cudaStream_t s)
{
    dot_kernel<T><<<red_grid(n), kRedThreads, 0, s>>>(n, x, y, c->red_partial, c->red_counter, out);
    SC_CHECK_LAUNCH();
    return 0;
}

template int dot_dev<double>(scalit_ctx *, i64, const double *, const double *, double *, cudaStream_t);
template int dot_dev<float>(scalit_ctx *, i64, const float *, const float *, double *, cudaStream_t);

// ------------------------------------------------------------------ driver --
// One QMR solve of nrhs right-hand sides (B, X: n x nrhs, column v at v n)
// advancing in lockstep: every vector kernel runs over all of them
// (blockIdx.y = v), each with its own scalar state, and the operators are
// applied to the whole block at once.  A right-hand side whose recurrence
// stopped is skipped by the vector kernels; the operators stop when all have.
template <class T>
int QmrSolve<T>::setup(scalit_ctx *ctx, i64 n_, int nrhs_, QmrOps<T> *ops_, int ntype_, int qmrmax_,
                       double tol_, const T *B, const T *X, cudaStream_t stream)
{
    c = ctx; n = n_; nrhs = nrhs_; ops = ops_; ntype = ntype_; qmrmax = qmrmax_; tol = tol_; s = stream;
    const i64 nn = n * nrhs;
    // vectors: R UX UR Q S V Z HX0, the right-hand sides and solution copies,
    // the preconditioner's scratch; then the states, the partial sums and the
    // all-stopped flag
    const size_t vec_bytes = sizeof(T) * (size_t)nn * 11;
    const size_t st_off = (vec_bytes + 255) & ~(size_t)255;
    const size_t part_off = (st_off + sizeof(QmrState) * (size_t)nrhs + 255) & ~(size_t)255;
    const size_t flag_off = part_off + sizeof(double) * (size_t)kPartStride * nrhs;
    const size_t need = flag_off + 64;
    unsigned char *w = nullptr;
    int rc = work_get(c, need, (void **)&w);
    if (rc) return rc;
    T *v = reinterpret_cast<T *>(w);
    R = v; UX = v + nn; UR = v + 2 * nn; Q = v + 3 * nn; S = v + 4 * nn; V = v + 5 * nn;
    Z = v + 6 * nn; HX0 = v + 7 * nn; Bw = v + 8 * nn; Xw = v + 9 * nn; Pt = v + 10 * nn;
    st = reinterpret_cast<QmrState *>(w + st_off);
    partial = reinterpret_cast<double *>(w + part_off);
    alldone = reinterpret_cast<int *>(w + flag_off);
    gate = (nrhs == 1) ? &st->done : alldone;
    gr = red_grid(n);
    ge = ew_grid(n);
    ops->set_scratch(Pt);

    QmrState h{};
    h.ZVRAT = 1.0;
    h.GAMAMO = 1.0;
    h.ETA = -1.0;
    h.i = 1;
    h.qmrmax = qmrmax;
    h.ntype = ntype;
    h.tol = tol;
    std::vector<QmrState> hs((size_t)nrhs, h);
    SC_CUDA(cudaMemcpyAsync(st, hs.data(), sizeof(QmrState) * (size_t)nrhs, cudaMemcpyHostToDevice, s));
    SC_CUDA(cudaMemsetAsync(alldone, 0, sizeof(int), s));
    SC_CUDA(cudaMemcpyAsync(Bw, B, sizeof(T) * (size_t)nn, cudaMemcpyDeviceToDevice, s));
    if (ntype <= 0) SC_CUDA(cudaMemsetAsync(Xw, 0, sizeof(T) * (size_t)nn, s));
    else SC_CUDA(cudaMemcpyAsync(Xw, X, sizeof(T) * (size_t)nn, cudaMemcpyDeviceToDevice, s));
    copy_kernel<T><<<ew_grid(nn), 256, 0, s>>>(nn, Bw, R, V);
    SC_CHECK_LAUNCH();
    rc = ops->px(Bw, Z, nullptr);
    if (rc) return rc;
    qmr_init_norms<T><<<dim3(gr, nrhs), kRedThreads, 0, s>>>(n, n, Bw, Z, st, partial);
    if (nrhs > 1) qmr_all_done<<<1, 32, 0, s>>>(st, nrhs, alldone);
    SC_CHECK_LAUNCH();
    return 0;
}

// One iteration; every launch is gated by the states' done flags.
template <class T>
int QmrSolve<T>::iteration()
{
    const dim3 gR(gr, nrhs), gE(ge, nrhs);
    qmr_step_a<T><<<gR, kRedThreads, 0, s>>>(n, n, V, Z, st, partial);
    qmr_step_b<T><<<gE, 256, 0, s>>>(n, n, Z, Q, st);
    SC_CHECK_LAUNCH();
    // S = (H - E0) Q; step C scales it by ZVRAT as the reference does
    int r = ops->hx(Q, S, gate);
    if (r) return r;
    qmr_step_c<T><<<gR, kRedThreads, 0, s>>>(n, n, Q, S, st, partial);
    qmr_step_d<T><<<gR, kRedThreads, 0, s>>>(n, n, S, V, st, partial);
    SC_CHECK_LAUNCH();
    r = ops->px(V, Z, gate);
    if (r) return r;
    qmr_step_e<T><<<gR, kRedThreads, 0, s>>>(n, n, Z, st, partial);
    qmr_step_f<T><<<gR, kRedThreads, 0, s>>>(n, n, Q, S, UX, UR, Xw, R, st, partial);
    SC_CHECK_LAUNCH();
    if (abs(ntype) == 1) {
        r = ops->hx(Xw, HX0, gate);
        if (r) return r;
        qmr_step_g<T><<<gR, kRedThreads, 0, s>>>(n, n, HX0, Bw, st, partial);
        SC_CHECK_LAUNCH();
    }
    if (nrhs > 1) {
        qmr_all_done<<<1, 32, 0, s>>>(st, nrhs, alldone);
        SC_CHECK_LAUNCH();
    }
    return 0;
}

template <class T>
int QmrSolve<T>::finish(T *X, QmrResult *out)
{
    std::vector<QmrState> hs((size_t)nrhs);
    SC_CUDA(cudaMemcpyAsync(hs.data(), st, sizeof(QmrState) * (size_t)nrhs, cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaMemcpyAsync(X, Xw, sizeof(T) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, s));
    SC_CUDA(cudaStreamSynchronize(s));
    for (int v = 0; v < nrhs; ++v) {
        out[v].code = hs[v].code;
        out[v].res = hs[v].RES;
        out[v].iters = hs[v].iters;
        out[v].breakdown = hs[v].breakdown;
    }
    return tc_check_error(c);
}

template <class T>
int qmr_core_n(scalit_ctx *c, i64 n, int nrhs, QmrOps<T> &ops, int ntype, int qmrmax, double qmrtol,
               const T *B, T *X, QmrResult *out)
{
    cudaStream_t s = c->stream;
    QmrSolve<T> q;
    int rc = q.setup(c, n, nrhs, &ops, ntype, qmrmax, qmrtol, B, X, s);
    if (rc) return rc;
    const int batch = ops.host_side() ? 1 : 4;
    // Device-side operators: the batch of iterations is captured once as a CUDA
    // graph per context and precision and replayed (all pointers live in the
    // workspace; the launches read their scalars from the device states).
    cudaGraphExec_t exec = nullptr, own_exec = nullptr;
    if (!ops.host_side() && nrhs > 1) {
        // several right-hand sides: the operators' shift arrays belong to this
        // call, so the graph is captured for it alone
        cudaGraph_t graph = nullptr;
        SC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int r = 0;
        for (int b = 0; b < batch && !r; ++b) r = q.iteration();
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (r) { if (graph) cudaGraphDestroy(graph); return r; }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
        const cudaError_t ie = cudaGraphInstantiate(&own_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate", __FILE__, __LINE__);
        exec = own_exec;
    } else if (!ops.host_side()) {
        scalit_ctx::QmrGraph &qg = c->qg[sizeof(T) == 8 ? 0 : 1];
        if (qg.exec && (qg.gen != c->gen || qg.ntype != ntype || qg.n != n || qg.work != c->work ||
                        qg.nrhs != nrhs)) {
            cudaGraphExecDestroy(qg.exec);
            qg.exec = nullptr;
        }
        if (!qg.exec) {
            cudaGraph_t graph = nullptr;
            SC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int r = 0;
            for (int b = 0; b < batch && !r; ++b) r = q.iteration();
            const cudaError_t ce = cudaStreamEndCapture(s, &graph);
            if (r) { if (graph) cudaGraphDestroy(graph); return r; }
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
            const cudaError_t ie = cudaGraphInstantiate(&qg.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) { qg.exec = nullptr; return cuda_fail(ie, "cudaGraphInstantiate", __FILE__, __LINE__); }
            qg.gen = c->gen;
            qg.ntype = ntype;
            qg.n = n;
            qg.work = c->work;
            qg.nrhs = nrhs;
        }
        exec = qg.exec;
    }

    int it = 0;
    int *h_flag = reinterpret_cast<int *>(c->h_pinned);
    while (rc == 0) {
        if (exec) {
            if (cudaGraphLaunch(exec, s) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "cudaGraphLaunch", __FILE__, __LINE__); break; }
        } else {
            for (int b = 0; b < batch && !rc; ++b) rc = q.iteration();
            if (rc) break;
        }
        it += batch;
        if (cudaMemcpyAsync(h_flag, q.gate, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "QMR poll", __FILE__, __LINE__); break; }
        if (*h_flag) break;
        if (it > qmrmax + batch) { set_error("QMR did not stop"); rc = SCALIT_ESTATE; }
    }
    if (own_exec) cudaGraphExecDestroy(own_exec);
    if (rc) return rc;
    return q.finish(X, out);
}

template <class T>
int qmr_core(scalit_ctx *c, i64 n, QmrOps<T> &ops, int ntype, int qmrmax, double qmrtol,
             const T *B, T *X, QmrResult *out)
{
    return qmr_core_n<T>(c, n, 1, ops, ntype, qmrmax, qmrtol, B, X, out);
}

template struct QmrSolve<double>;
template struct QmrSolve<float>;
template int qmr_core_n<double>(scalit_ctx *, i64, int, QmrOps<double> &, int, int, double, const double *, double *, QmrResult *);
template int qmr_core_n<float>(scalit_ctx *, i64, int, QmrOps<float> &, int, int, double, const float *, float *, QmrResult *);
template int qmr_core<double>(scalit_ctx *, i64, QmrOps<double> &, int, int, double, const double *, double *, QmrResult *);
template int qmr_core<float>(scalit_ctx *, i64, QmrOps<float> &, int, int, double, const float *, float *, QmrResult *);

// The context's own operator pair: HX = MYHX(TA1), PX = MYPX(sOSB, TA1).
template <class T> struct CtxQmrOps : QmrOps<T> {
    scalit_ctx *c;
    T *tmp = nullptr;
    void set_scratch(T *p) override { tmp = p; }
    int hx(const T *in, T *out, const int *gate) override
    {
        return hx_vec<T>(c, in, out, T(c->E0), T(1), gate, c->stream);
    }
    int px(const T *in, T *out, const int *gate) override
    {
        return px_vec<T>(c, SCALIT_TA1, in, out, tmp, T(1), gate, c->stream);
    }
};

// Mixed-precision iterative refinement around the FP32 QMR: X = 0, r = B;
// each round solves (H - E0) d = r in FP32 (the context's FP32 operators, the
// QMR's own test with tolerance max(1e-4, qmrtol |B - r| / |r|), x0 = 0),
// adds d to X in FP64 and forms r = B - (H - E0) X with an FP64 H*X.  It stops
// when |r| <= qmrtol |B - r| (the type -1 measure |HX - B| / |HX| in FP64),
// after 5 rounds, or when the rounds have used qmrmax iterations.  The code
// is the total iteration count, negated when the tolerance was not reached;
// an FP32 round that breaks down ends the solve with its code.
static int qmr_refined(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, const double *dB, double *dX,
                       QmrResult *out)
{
    const i64 n = c->L.N;
    cudaStream_t s = c->stream;
    double *r = nullptr, *d = nullptr, *dd = nullptr;
    float *bx = nullptr;
    int rc = 0;
    if (cudaMallocAsync(&r, sizeof(double) * (size_t)n, s) != cudaSuccess ||
        cudaMallocAsync(&d, sizeof(double) * (size_t)n, s) != cudaSuccess ||
        cudaMallocAsync(&dd, sizeof(double) * 4, s) != cudaSuccess ||
        cudaMallocAsync(&bx, sizeof(float) * 2 * (size_t)n, s) != cudaSuccess) {
        cudaGetLastError();
        set_error("refined QMR workspace does not fit");
        rc = SCALIT_ENOMEM;
    }
    auto norm2 = [&](const double *x, double *h) -> int {
        int e = dot_dev<double>(c, n, x, x, dd, s);
        if (!e) e = sync_read_doubles(c, dd, h, 1);
        return e;
    };
    double nb = 0.0;
    if (!rc) rc = norm2(dB, &nb);
    if (!rc && cudaMemsetAsync(dX, 0, sizeof(double) * (size_t)n, s) != cudaSuccess) rc = SCALIT_ECUDA;
    if (!rc && cudaMemcpyAsync(r, dB, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        rc = SCALIT_ECUDA;
    QmrResult res{};
    int total = 0;
    bool converged = false;
    double rel = 1.0, nr2 = nb;
    CtxQmrOps<float> ops;
    ops.c = c;
    for (int round = 0; round < 5 && !rc && !converged && total < qmrmax; ++round) {
        if (nr2 == 0.0) { converged = true; break; }
        const double tin = std::min(0.5, std::max(1e-4, qmrtol / std::max(rel, 1e-300)));
        QmrResult q{};
        rc = to_f32(r, bx, n, s);
        if (!rc) rc = qmr_core<float>(c, n, ops, ntype > 0 ? -1 : ntype, qmrmax - total, tin, bx, bx + n, &q);
        if (rc) break;
        total += q.iters;
        res.breakdown = q.breakdown;
        if (q.breakdown) { res.code = q.code; break; }
        rc = to_f64(bx + n, d, n, s);
        if (!rc) rc = axpy_dev(n, 1.0, d, dX, s);
        // r = B - (H - E0) X in FP64
        if (!rc) rc = hx_vec<double>(c, dX, r, c->E0, -1.0, nullptr, s);
        if (!rc) rc = axpy_dev(n, 1.0, dB, r, s);
        double hx2 = 0.0;
        if (!rc) rc = norm2(r, &nr2);
        if (rc) break;
        // |HX|^2 = |B - r|^2
        if (cudaMemcpyAsync(d, dB, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            rc = SCALIT_ECUDA;
            break;
        }
        rc = axpy_dev(n, -1.0, r, d, s);
        if (!rc) rc = norm2(d, &hx2);
        if (rc) break;
        rel = (hx2 > 0.0) ? std::sqrt(nr2 / hx2) : 1.0;
        res.res = rel;
        converged = rel <= qmrtol;
    }
    if (!rc && !res.breakdown) res.code = converged ? std::max(total, 1) : -std::max(total, 1);
    res.iters = total;
    if (r) cudaFreeAsync(r, s);
    if (d) cudaFreeAsync(d, s);
    if (dd) cudaFreeAsync(dd, s);
    if (bx) cudaFreeAsync(bx, s);
    if (!rc && out) *out = res;
    return rc;
}

int qmr_run(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision,
            const double *dB, double *dX, QmrResult *out)
{
    if (!c->osb_built) { set_error("QMR needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
    const i64 n = c->L.N;
    if (precision == SCALIT_PREC_FP64) {
        CtxQmrOps<double> ops;
        ops.c = c;
        return qmr_core<double>(c, n, ops, ntype, qmrmax, qmrtol, dB, dX, out);
    }
    if (precision == SCALIT_PREC_FP32_REFINED) return qmr_refined(c, ntype, qmrmax, qmrtol, dB, dX, out);
    if (precision != SCALIT_PREC_FP32) { set_error("unknown precision %d", precision); return SCALIT_EINVAL; }
    float *bx = nullptr;
    SC_CUDA(cudaMallocAsync(&bx, sizeof(float) * 2 * (size_t)n, c->stream));
    CtxQmrOps<float> ops;
    ops.c = c;
    int rc = to_f32(dB, bx, n, c->stream);
    if (!rc) rc = qmr_core<float>(c, n, ops, ntype, qmrmax, qmrtol, bx, bx + n, out);
    if (!rc) rc = to_f64(bx + n, dX, n, c->stream);
    cudaFreeAsync(bx, c->stream);
    return rc;
}

}  // namespace sc
