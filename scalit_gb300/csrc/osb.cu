// OSB preconditioner build: layered joint block-Jacobi diagonalisation.
//
// myDiag (src/iterate/module/osb.diag.h:53-151) runs, for level = sF..1,
//   HOSBINIT_DEP / HOSBINIT_XYZ (src/iterate/libiterate/diag/hinitdep.f90:10-34,
//   hinitxyz.f90:7-29):  HOSB(k, r, c, b) = H(r, c) [* DEP(k)] + delta_rc EIG0(k, r, b)
// and then HosbDiag (hosbdiag.f90:5-75): sweeps of joint Jacobi rotations over
// the (p, q) planes in the order  i = 1..MAK-1, j = 1..MAK-i, (p, q) = (j, j+i),
// each rotation's angle taken from A = sum_k o^2, B = 2 sum_k o d, C = sum_k d^2
// (MJACOBI, jacobi.f90:2-83), V accumulated by VUPDATE (vupdate.f90:21-36),
// until |change of sumOffDiag| <= BJTOL * initial or BJMAX sweeps; EIG0 takes
// the rotated diagonal and the diagonal of HOSB is zeroed.
//
// The rotation order is the reference's, so V and EIG0 agree with it to
// rounding.  Within one offset i the rotations (j, j+i), (j+1, j+1+i), ...,
// (j+m-1, j+m-1+i) with m <= i act on disjoint planes: none of them changes an
// element another one reads for its angle, so their angles are the ones the
// sequential order computes, and each element is touched by at most two of
// them, applied here in the sequential order.  A sweep therefore runs as
// about MAK ln MAK batches instead of MAK (MAK-1) / 2 single rotations.  Two
// device schedules:
//  * the block's stacked matrices fit in shared memory (level 1: one n x n
//    matrix per block): one CTA per block runs all its sweeps in SMEM;
//  * otherwise (the outer levels' stacks of NDK matrices): every batch is
//    spread over the whole GPU and all blocks -- one launch forms the batch's
//    angles and rotates V, a second rotates HOSB.
// The angle is formed from A, B, C with square roots only (half-angle
// identities for atan(B/(A-C))/4 and the +-pi/4 shifts), which equals the
// reference's DATAN/DSIN/DCOS result to rounding.
#include "internal.cuh"

#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <type_traits>
#include <vector>

namespace sc {

static constexpr int kThreads = 256;

// cos and sin of the MJACOBI angle (jacobi.f90:42-60), in the precision of
// the sweep (FP64, or FP32 for a preconditioner built in single precision).
template <typename R>
__device__ void jacobi_angle(R A, R B, R C, R *cs, R *sn)
{
    const R INV_SQRT2 = R(0.70710678118654752440), one = R(1), half = R(0.5), two = R(2);
    if (A == C) {
        if (B == R(0)) { *cs = one; *sn = R(0); return; }
        // X = -sign(pi/8, B)
        const R c8 = sqrt(half * (one + INV_SQRT2));
        const R s8 = sqrt(half * (one - INV_SQRT2));
        *cs = c8;
        *sn = (B > R(0)) ? -s8 : s8;
        return;
    }
    const R T = B / (A - C);
    R c4, s4;   // cos, sin of atan(T)
    if (fabs(T) > one) {
        const R r = one / T;
        const R h = sqrt(one + r * r);
        c4 = fabs(r) / h;
        s4 = (T > R(0) ? one : -one) / h;
    } else {
        c4 = one / sqrt(one + T * T);
        s4 = T * c4;
    }
    const R c2 = sqrt(half * (one + c4));
    const R s2 = s4 / (two * c2);
    R c = sqrt(half * (one + c2));
    R s = s2 / (two * c);
    if (A > C) {
        R nc, ns;
        if (s < R(0)) {       // X + pi/4  (X < 0 <=> s < 0)
            nc = (c - s) * INV_SQRT2;
            ns = (s + c) * INV_SQRT2;
        } else {              // X - pi/4
            nc = (c + s) * INV_SQRT2;
            ns = (s - c) * INV_SQRT2;
        }
        c = nc;
        s = ns;
    }
    *cs = c;
    *sn = s;
}

// Deterministic block-wide sum of three values; result broadcast to all threads.
__device__ void block_sum3(double &a, double &b, double &c, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    __syncthreads();
    if (lane == 0) { red[3 * warp] = a; red[3 * warp + 1] = b; red[3 * warp + 2] = c; }
    __syncthreads();
    a = 0.0; b = 0.0; c = 0.0;
    for (int w = 0; w < nw; ++w) { a += red[3 * w]; b += red[3 * w + 1]; c += red[3 * w + 2]; }
}

// Reductions over one block's stacked matrices; element (k, r, c) of the
// stack sits at k + ndk (r + ldr c) (ldr = MAK, or MAK + 1 in shared memory
// where the padding keeps row and column walks free of bank conflicts).
__device__ double block_offdiag(const double *H, int ndk, int mak, int ldr, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    const int per_col = ndk * mak;
    for (int col = 1; col < mak; ++col) {
        const int cnt = ndk * col;                 // rows 0..col-1 of every stacked matrix
        const double *Hc = H + (i64)ndk * ldr * col;
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) { const double h = Hc[e]; s = fma(h, h, s); }
    }
    (void)per_col;
    block_sum3(s, z1, z2, red);
    return 2.0 * s;
}

__device__ double block_sumdiag(const double *H, int ndk, int mak, int ldr, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    const int total = ndk * mak;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int i = e / ndk, k = e - i * ndk;
        const double h = H[k + (i64)ndk * (i + (i64)ldr * i)];
        s = fma(h, h, s);
    }
    block_sum3(s, z1, z2, red);
    return s;
}

// A batch: planes t = 0..m-1, (p_t, q_t) = (a + t, a + i + t), m <= i.
// Its HOSB work items per stacked matrix: (MAK - 2m) * m pair updates of a row
// outside the batch's planes, then an m x m grid of (t, t2) 2x2 blocks (t == t2:
// the plane's own diagonal block; t < t2: the cross block, rotation t first).
__host__ __device__ __forceinline__ int batch_items(int mak, int m)
{
    return (mak - 2 * m) * m + m * m;
}

// u / m and u % m for 0 <= u < 2^24, 1 <= m and a quotient below 2^20, from
// rm = 1 / m in FP32: the product is then off by less than one, which the
// single correction step fixes (integer division costs tens of instructions).
__device__ __forceinline__ int quot_small(int u, int m, float rm, int &rem)
{
    int q = __float2int_rz(__int2float_rn(u) * rm);
    int r = u - q * m;
    if (r < 0) { --q; r += m; }
    else if (r >= m) { ++q; r -= m; }
    rem = r;
    return q;
}

__device__ __forceinline__ int free_row(int f, int a, int i, int m)
{
    if (f < a) return f;
    f -= a;
    if (f < i - m) return a + m + f;
    return a + i + m + (f - (i - m));
}

// MJACOBI's update (jacobi.f90:62-80) of work item u of stacked matrix k.
// ONE: a single matrix per block (ndk == 1) with 32-bit offsets.
template <bool ONE, typename R = double>
__device__ __forceinline__ void batch_item(R *H, int ndk_, int mak, int ldr, int a, int i, int m,
                                           const double *__restrict__ cs, const double *__restrict__ sn,
                                           int u, int k, float rm)
{
    using I = typename std::conditional<ONE, int, i64>::type;
    const I ndk = ONE ? 1 : (I)ndk_;
    const int nfree = (mak - 2 * m) * m;
    const I ld = ndk * (I)ldr;
    R *Hk = H + (ONE ? 0 : k);
    if (u < nfree) {
        int t;
        const int f = quot_small(u, m, rm, t), r = free_row(f, a, i, m);
        const int p = a + t, q = a + i + t;
        R *hrp = Hk + ndk * r + ld * p, *hrq = Hk + ndk * r + ld * q;
        R *hpr = Hk + ndk * p + ld * r, *hqr = Hk + ndk * q + ld * r;
        const R c = (R)cs[t], sv = (R)sn[t];
        const R x = *hrp, y = *hrq;
        const R np_ = c * x - sv * y;
        const R nq_ = c * y + sv * x;
        *hrp = np_; *hpr = np_; *hrq = nq_; *hqr = nq_;
        return;
    }
    u -= nfree;
    int t2;
    const int t = quot_small(u, m, rm, t2);
    if (t2 < t) return;
    const int p = a + t, q = a + i + t;
    const R c = (R)cs[t], sv = (R)sn[t];
    if (t == t2) {
        R *hpp = Hk + ndk * p + ld * p, *hqq = Hk + ndk * q + ld * q;
        R *hpq = Hk + ndk * p + ld * q, *hqp = Hk + ndk * q + ld * p;
        const R C2 = c * c, S2 = sv * sv, SC = sv * c;
        const R odg = *hpq;
        const R ddg = R(0.5) * *hpp - R(0.5) * *hqq;
        const R np_ = C2 * *hpp + S2 * *hqq - R(2) * SC * odg;
        const R nq_ = C2 * *hqq + S2 * *hpp + R(2) * SC * odg;
        const R nqp = (C2 - S2) * odg + R(2) * SC * ddg;
        *hpp = np_; *hqq = nq_; *hpq = nqp; *hqp = nqp;
        return;
    }
    const int p2 = a + t2, q2 = a + i + t2;
    R *h00 = Hk + ndk * p + ld * p2, *h01 = Hk + ndk * p + ld * q2;
    R *h10 = Hk + ndk * q + ld * p2, *h11 = Hk + ndk * q + ld * q2;
    // rotation t acts on rows p2 and q2 as rows outside its plane ...
    const R x00 = *h00, x01 = *h01, x10 = *h10, x11 = *h11;
    const R a00 = c * x00 - sv * x10, a10 = c * x10 + sv * x00;
    const R a01 = c * x01 - sv * x11, a11 = c * x11 + sv * x01;
    // ... then rotation t2 on rows p and q
    const R c2 = (R)cs[t2], s2 = (R)sn[t2];
    const R b00 = c2 * a00 - s2 * a01, b01 = c2 * a01 + s2 * a00;
    const R b10 = c2 * a10 - s2 * a11, b11 = c2 * a11 + s2 * a10;
    *h00 = b00; *h01 = b01; *h10 = b10; *h11 = b11;
    Hk[ndk * p2 + ld * p] = b00; Hk[ndk * q2 + ld * p] = b01;
    Hk[ndk * p2 + ld * q] = b10; Hk[ndk * q2 + ld * q] = b11;
}

// VUPDATE (vupdate.f90:21-36) of item u = (t, row), rows fastest: columns
// p_t, q_t of V.
template <typename R>
__device__ __forceinline__ void batch_vitem(R *V, int mak, int a, int i,
                                            const R *__restrict__ cs, const R *__restrict__ sn,
                                            int u, float rmak)
{
    int row;
    const int t = quot_small(u, mak, rmak, row);
    R *vp = V + (i64)(a + t) * mak + row, *vq = V + (i64)(a + i + t) * mak + row;
    const R c = cs[t], sv = sn[t];
    const R x = *vp, y = *vq;
    *vp = c * x - sv * y;
    *vq = c * y + sv * x;
}

// ------------------------------------------------------------------ init --
__global__ void hosb_init_kernel(int blk, int mak, int ndk, const double *__restrict__ H1,
                                 const double *__restrict__ DEP, const double *__restrict__ RES,
                                 double *__restrict__ HOSB)
{
    const i64 total = (i64)ndk * mak * mak * blk;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int k = (int)(e % ndk);
        i64 t = e / ndk;
        const int r = (int)(t % mak); t /= mak;
        const int c = (int)(t % mak);
        const i64 b = t / mak;
        double v = H1[r + (i64)mak * c];
        if (DEP) v = v * DEP[k];
        if (r == c) v = v + RES[k + (i64)ndk * (r + (i64)mak * b)];
        HOSB[e] = v;
    }
}

// ------------------------------------------------- schedule 1: CTA/block --
static constexpr int kMaxBatch = 128;   // m <= MAK / 2
// Large blocks leave room for one CTA per SM (the block's matrix fills shared
// memory), so that CTA brings the warps that hide the FP64 pipe's and shared
// memory's latencies: up to 1024 threads.
static constexpr int kJacThreads = 1024;

__global__ void __launch_bounds__(kJacThreads, 1)
jacobi_block_kernel(int bjmax, double bjtol, int blk, int mak, int ndk,
                    double *__restrict__ HOSB, double *__restrict__ VOSB, double *__restrict__ EIG,
                    double *__restrict__ bstats)
{
    extern __shared__ __align__(16) double smem[];
    double *red = smem;                 // 3 * 32
    double *cs = smem + 96;             // kMaxBatch
    double *sn = cs + kMaxBatch;        // kMaxBatch
    double *abc_c = sn + kMaxBatch;     // kMaxBatch (C sums of a stacked batch)
    double *cs_v = abc_c + kMaxBatch;   // kMaxBatch: the previous batch's angles, for
    double *sn_v = cs_v + kMaxBatch;    // kMaxBatch  its deferred V update (one matrix)
    double *H = sn_v + kMaxBatch;       // the block's stacked matrices, column stride ldr
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    const int ldr = (ndk == 1) ? mak + 1 : mak;
    const int col_g = ndk * mak, col_s = ndk * ldr;     // one column of the stack: global / shared
    const float rmak = 1.0f / (float)mak;
    for (int b = blockIdx.x; b < blk; b += gridDim.x) {
        double *Hg = HOSB + (i64)b * col_g * mak;
        double *V = VOSB + (i64)b * mak * mak;
        __syncthreads();
        for (int c = 0; c < mak; ++c)
            for (int e = tid; e < col_g; e += nt) H[e + c * col_s] = Hg[e + (i64)c * col_g];
        for (int e = tid; e < mak * mak; e += nt) { const int c = e / mak; V[e] = (e - c * mak == c) ? 1.0 : 0.0; }
        __syncthreads();
        const double initye = block_offdiag(H, ndk, mak, ldr, red);
        double ye = initye, dye = initye;
        int k = 1;
        // one matrix: a batch's V update waits for the next batch's angle
        // phase, so the FP64 pipe works on V while a few threads run the
        // angles' divisions and square roots (V does not feed the angles)
        int mv = 0, av = 0, iv = 0;
        while (fabs(dye) > initye * bjtol && k <= bjmax) {
            for (int i = 1; i <= mak - 1; ++i) {
                for (int a = 0; a < mak - i; a += i) {
                    const int m = min(i, mak - i - a);
                    // angles of the batch: one thread per plane (the FP64 square
                    // roots and divisions then fill whole warps); with a stack of
                    // matrices one warp per plane first sums A, B, C over it
                    if (ndk == 1) {
                        const int t0 = (m + 31) & ~31;          // warps past the angle threads
                        if (tid < m) {
                            const int p = a + tid, q = a + i + tid;
                            const double o = H[p + ldr * q];
                            const double d = 0.5 * H[p + ldr * p] - 0.5 * H[q + ldr * q];
                            jacobi_angle(o * o, 2.0 * (o * d), d * d, cs + tid, sn + tid);
                        } else if (tid >= t0) {                 // t0 <= kMaxBatch < nt
                            for (int u = tid - t0; u < mak * mv; u += nt - t0)
                                batch_vitem(V, mak, av, iv, cs_v, sn_v, u, rmak);
                        }
                    } else {
                        for (int t = warp; t < m; t += nw) {
                            const int p = a + t, q = a + i + t;
                            double sA = 0.0, sB = 0.0, sC = 0.0;
                            for (int kk = lane; kk < ndk; kk += 32) {
                                const double o = H[kk + ndk * (p + ldr * q)];
                                const double d = 0.5 * H[kk + ndk * (p + ldr * p)]
                                               - 0.5 * H[kk + ndk * (q + ldr * q)];
                                sA = fma(o, o, sA); sB = fma(o, d, sB); sC = fma(d, d, sC);
                            }
                            #pragma unroll
                            for (int o = 16; o > 0; o >>= 1) {
                                sA += __shfl_xor_sync(0xffffffffu, sA, o);
                                sB += __shfl_xor_sync(0xffffffffu, sB, o);
                                sC += __shfl_xor_sync(0xffffffffu, sC, o);
                            }
                            if (lane == 0) { cs[t] = sA; sn[t] = sB; abc_c[t] = sC; }
                        }
                        __syncthreads();
                        for (int t = tid; t < m; t += nt) jacobi_angle(cs[t], 2.0 * sn[t], abc_c[t], cs + t, sn + t);
                    }
                    __syncthreads();
                    const int nh = batch_items(mak, m);
                    const float rm = 1.0f / (float)m;
                    if (ndk == 1) {
                        for (int u = tid; u < nh; u += nt) batch_item<true>(H, 1, mak, ldr, a, i, m, cs, sn, u, 0, rm);
                        // keep this batch's angles for its V update
                        if (tid < m) { cs_v[tid] = cs[tid]; sn_v[tid] = sn[tid]; }
                        mv = m; av = a; iv = i;
                    } else {
                        for (int e = tid; e < ndk * nh; e += nt) {
                            const int u = e / ndk;
                            batch_item<false>(H, ndk, mak, ldr, a, i, m, cs, sn, u, e - u * ndk, rm);
                        }
                        for (int u = tid; u < mak * m; u += nt) batch_vitem(V, mak, a, i, cs, sn, u, rmak);
                    }
                    __syncthreads();
                }
            }
            dye = block_offdiag(H, ndk, mak, ldr, red) - ye;
            ye = ye + dye;
            k = k + 1;
        }
        // the last batch's V update
        for (int u = tid; u < mak * mv; u += nt) batch_vitem(V, mak, av, iv, cs_v, sn_v, u, rmak);
        const double sd = block_sumdiag(H, ndk, mak, ldr, red);
        __syncthreads();
        for (int e = tid; e < ndk * mak; e += nt) {
            const int i = e / ndk, kk = e - i * ndk;
            const int di = kk + ndk * (i + ldr * i);
            EIG[kk + (i64)ndk * (i + (i64)mak * b)] = H[di];
            H[di] = 0.0;
        }
        __syncthreads();
        for (int c = 0; c < mak; ++c)
            for (int e = tid; e < col_g; e += nt) Hg[e + (i64)c * col_g] = H[e + c * col_s];
        if (tid == 0) {
            bstats[3 * (i64)b] = (double)k;
            bstats[3 * (i64)b + 1] = fabs(1.0 - ye / initye);
            bstats[3 * (i64)b + 2] = sd;
        }
    }
}

// ------------------------------------- schedule 1b: CTA/block, packed --
// One matrix per block (ndk == 1) kept as its upper triangle, column by
// column (element (r, c), r <= c, at c (c + 1) / 2 + r): half the shared
// memory of the full square, so two 160 x 160 blocks fit an SM and one CTA's
// angle phases and barriers overlap the other's rotations.  Every element
// update is the full-storage kernel's (the same formulas on the same values,
// one stored copy instead of two mirrored ones), so H, V and the
// eigenvalues evolve bit for bit alike; only the order of the sweep
// reductions' sums differs.
__device__ __forceinline__ int pk(int r, int c) { return ((c * (c + 1)) >> 1) + r; }   // r <= c
__device__ __forceinline__ int pks(int a, int b) { return a <= b ? pk(a, b) : pk(b, a); }

template <typename R>
__device__ __forceinline__ void packed_item(R *H, int mak, int a, int i, int m,
                                            const R *__restrict__ cs, const R *__restrict__ sn,
                                            int u, float rm)
{
    const int nfree = (mak - 2 * m) * m;
    if (u < nfree) {
        int t;
        const int f = quot_small(u, m, rm, t), r = free_row(f, a, i, m);
        const int p = a + t, q = a + i + t;
        const int ip = pks(r, p), iq = pks(r, q);
        const R c = cs[t], sv = sn[t];
        const R x = H[ip], y = H[iq];
        H[ip] = c * x - sv * y;
        H[iq] = c * y + sv * x;
        return;
    }
    u -= nfree;
    int t2;
    const int t = quot_small(u, m, rm, t2);
    if (t2 < t) return;
    const int p = a + t, q = a + i + t;
    const R c = cs[t], sv = sn[t];
    if (t == t2) {
        const int pp = pk(p, p), qq = pk(q, q), pq = pk(p, q);
        const R C2 = c * c, S2 = sv * sv, SC = sv * c;
        const R odg = H[pq];
        const R ddg = R(0.5) * H[pp] - R(0.5) * H[qq];
        const R np_ = C2 * H[pp] + S2 * H[qq] - R(2) * SC * odg;
        const R nq_ = C2 * H[qq] + S2 * H[pp] + R(2) * SC * odg;
        const R nqp = (C2 - S2) * odg + R(2) * SC * ddg;
        H[pp] = np_; H[qq] = nq_; H[pq] = nqp;
        return;
    }
    const int p2 = a + t2, q2 = a + i + t2;
    const int i00 = pks(p, p2), i01 = pks(p, q2), i10 = pks(q, p2), i11 = pks(q, q2);
    const R x00 = H[i00], x01 = H[i01], x10 = H[i10], x11 = H[i11];
    const R a00 = c * x00 - sv * x10, a10 = c * x10 + sv * x00;
    const R a01 = c * x01 - sv * x11, a11 = c * x11 + sv * x01;
    const R c2 = cs[t2], s2 = sn[t2];
    H[i00] = c2 * a00 - s2 * a01;
    H[i01] = c2 * a01 + s2 * a00;
    H[i10] = c2 * a10 - s2 * a11;
    H[i11] = c2 * a11 + s2 * a10;
}

// 2 sum over r < c of H(r, c)^2 and sum of H(c, c)^2, column by column
// (summed in FP64 for either element type).
template <typename R>
__device__ double packed_offdiag(const R *H, int mak, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    for (int c = 1; c < mak; ++c) {
        const R *Hc = H + pk(0, c);
        for (int r = threadIdx.x; r < c; r += blockDim.x) { const double h = Hc[r]; s = fma(h, h, s); }
    }
    block_sum3(s, z1, z2, red);
    return 2.0 * s;
}

template <typename R>
__device__ double packed_sumdiag(const R *H, int mak, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    for (int c = threadIdx.x; c < mak; c += blockDim.x) { const double h = H[pk(c, c)]; s = fma(h, h, s); }
    block_sum3(s, z1, z2, red);
    return s;
}

// R = float: the sweeps of a preconditioner built in single precision (its
// products only feed FP32 inner solves): H, the angles and V in FP32 (V in
// the first half of the block's FP64 storage, widened in place at the end),
// the sweep sums, EIG0 and the rotated HOSB in FP64.
template <typename R>
__global__ void __launch_bounds__(512, 2)
jacobi_packed_kernel(int bjmax, double bjtol, int blk, int mak, double *__restrict__ HOSB,
                     double *__restrict__ VOSB, double *__restrict__ EIG, double *__restrict__ bstats)
{
    extern __shared__ __align__(16) double smem[];
    double *red = smem;                 // 3 * 32
    R *cs = reinterpret_cast<R *>(smem + 96);   // kMaxBatch
    R *sn = cs + kMaxBatch;             // kMaxBatch
    R *cs_v = sn + kMaxBatch;           // kMaxBatch: the previous batch's angles, for
    R *sn_v = cs_v + kMaxBatch;         // kMaxBatch  its deferred V update
    R *H = sn_v + kMaxBatch;            // upper triangle, mak (mak + 1) / 2
    const int tid = threadIdx.x, nt = blockDim.x;
    const float rmak = 1.0f / (float)mak;
    for (int b = blockIdx.x; b < blk; b += gridDim.x) {
        double *Hg = HOSB + (i64)b * mak * mak;
        R *V = reinterpret_cast<R *>(VOSB + (i64)b * mak * mak);
        __syncthreads();
        for (int e = tid; e < mak * mak; e += nt) {
            int r;
            const int c = quot_small(e, mak, rmak, r);
            if (r <= c) H[pk(r, c)] = (R)Hg[e];
            V[e] = (r == c) ? R(1) : R(0);
        }
        __syncthreads();
        const double initye = packed_offdiag(H, mak, red);
        double ye = initye, dye = initye;
        int k = 1;
        int mv = 0, av = 0, iv = 0;
        while (fabs(dye) > initye * bjtol && k <= bjmax) {
            for (int i = 1; i <= mak - 1; ++i) {
                for (int a = 0; a < mak - i; a += i) {
                    const int m = min(i, mak - i - a);
                    // angles (one thread per plane) while the warps past them
                    // apply the previous batch's rotations to V
                    const int t0 = (m + 31) & ~31;          // t0 <= kMaxBatch < nt
                    if (tid < m) {
                        const int p = a + tid, q = a + i + tid;
                        const R o = H[pk(p, q)];
                        const R d = R(0.5) * H[pk(p, p)] - R(0.5) * H[pk(q, q)];
                        jacobi_angle(o * o, R(2) * (o * d), d * d, cs + tid, sn + tid);
                    } else if (tid >= t0) {
                        for (int u = tid - t0; u < mak * mv; u += nt - t0)
                            batch_vitem(V, mak, av, iv, cs_v, sn_v, u, rmak);
                    }
                    __syncthreads();
                    const int nh = batch_items(mak, m);
                    const float rm = 1.0f / (float)m;
                    for (int u = tid; u < nh; u += nt) packed_item(H, mak, a, i, m, cs, sn, u, rm);
                    if (tid < m) { cs_v[tid] = cs[tid]; sn_v[tid] = sn[tid]; }
                    mv = m; av = a; iv = i;
                    __syncthreads();
                }
            }
            dye = packed_offdiag(H, mak, red) - ye;
            ye = ye + dye;
            k = k + 1;
        }
        for (int u = tid; u < mak * mv; u += nt) batch_vitem(V, mak, av, iv, cs_v, sn_v, u, rmak);
        const double sd = packed_sumdiag(H, mak, red);
        __syncthreads();
        for (int e = tid; e < mak; e += nt) EIG[e + (i64)mak * b] = (double)H[pk(e, e)];
        // the rotated matrix back in full storage, its diagonal zeroed (as HOSB after HosbDiag)
        for (int e = tid; e < mak * mak; e += nt) {
            int r;
            const int c = quot_small(e, mak, rmak, r);
            Hg[e] = (r == c) ? 0.0 : (double)H[pks(r, c)];
        }
        if constexpr (sizeof(R) == sizeof(float)) {
            // widen V in place, last chunk of nt elements first: element e's
            // double covers floats 2e and 2e + 1, which belong to chunks
            // already read (or, for the first chunk, to itself and the next)
            double *Vd = VOSB + (i64)b * mak * mak;
            const int n = mak * mak;
            for (int j0 = ((n - 1) / nt) * nt; j0 >= 0; j0 -= nt) {
                const int e = j0 + tid;
                const float v = e < n ? V[e] : 0.0f;
                __syncthreads();
                if (e < n) Vd[e] = (double)v;
                __syncthreads();
            }
        }
        if (tid == 0) {
            bstats[3 * (i64)b] = (double)k;
            bstats[3 * (i64)b + 1] = fabs(1.0 - ye / initye);
            bstats[3 * (i64)b + 2] = sd;
        }
    }
}

// --------------------------------------------- schedule 2: GPU/rotation --
// Per-block state of the sweep loop: [initye, ye, dye, k, done, sumdiag].
struct SweepState { double initye, ye, dye; int k, done; double sumdiag; };

// R: the element type of the stacked matrices (FP64, or FP32 for a
// preconditioner built in single precision); sums, angles and V in FP64.
template <typename R>
__global__ void __launch_bounds__(kThreads)
gpu_partial_kernel(int mode, int mak, int ndk, const R *__restrict__ HOSB, double *__restrict__ partial)
{
    // mode 1: sumOffDiag; mode 2: sumDiag.
    __shared__ double red[96];
    const int b = blockIdx.y;
    const R *H = HOSB + (i64)b * ndk * mak * mak;
    double sA = 0.0, sB = 0.0, sC = 0.0;
    if (mode == 1) {
        // upper triangles: column col holds rows 0..col-1 contiguously (ndk * col numbers)
        for (int col = 1 + blockIdx.x; col < mak; col += gridDim.x) {
            const R *Hc = H + (i64)ndk * mak * col;
            const int cnt = ndk * col;
            for (int e = threadIdx.x; e < cnt; e += blockDim.x) { const double h = Hc[e]; sA = fma(h, h, sA); }
        }
    } else {
        const int total = ndk * mak;
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
            const int i = e / ndk, kk = e - i * ndk;
            const double h = H[kk + (i64)ndk * (i + (i64)mak * i)];
            sA = fma(h, h, sA);
        }
    }
    block_sum3(sA, sB, sC, red);
    if (threadIdx.x == 0) {
        double *out = partial + 3 * ((i64)b * gridDim.x + blockIdx.x);
        out[0] = sA; out[1] = sB; out[2] = sC;
    }
}

// One CTA per (plane t of the batch, block b): A, B, C over the stack, the
// angle, and V's columns p_t, q_t.
template <typename R>
__global__ void __launch_bounds__(kThreads)
gpu_batch_angle_kernel(int mak, int ndk, int a, int i, int blk, int ms, const R *__restrict__ HOSB,
                       double *__restrict__ rcs, double *__restrict__ rsn, double *__restrict__ VOSB,
                       const SweepState *__restrict__ st)
{
    __shared__ double red[96];
    __shared__ double cssn[2];
    const int t = blockIdx.x, p = a + t, q = a + i + t;
    for (int b = blockIdx.y; b < blk; b += gridDim.y) {
        if (st[b].done) continue;
        const R *H = HOSB + (i64)b * ndk * mak * mak;
        double sA = 0.0, sB = 0.0, sC = 0.0;
        for (int kk = threadIdx.x; kk < ndk; kk += blockDim.x) {
            const double o = H[kk + (i64)ndk * (p + (i64)mak * q)];
            const double d = 0.5 * H[kk + (i64)ndk * (p + (i64)mak * p)]
                           - 0.5 * H[kk + (i64)ndk * (q + (i64)mak * q)];
            sA = fma(o, o, sA); sB = fma(o, d, sB); sC = fma(d, d, sC);
        }
        block_sum3(sA, sB, sC, red);
        if (threadIdx.x == 0) {
            double c, sv;
            jacobi_angle(sA, 2.0 * sB, sC, &c, &sv);
            cssn[0] = c; cssn[1] = sv;
            rcs[(i64)b * ms + t] = c;
            rsn[(i64)b * ms + t] = sv;
        }
        __syncthreads();
        const double c = cssn[0], sv = cssn[1];
        double *V = VOSB + (i64)b * mak * mak;
        for (int row = threadIdx.x; row < mak; row += blockDim.x) {
            double *vp = V + (i64)p * mak + row, *vq = V + (i64)q * mak + row;
            const double x = *vp, y = *vq;
            *vp = c * x - sv * y;
            *vq = c * y + sv * x;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kThreads)
gpu_batch_rotate_kernel(int mak, int ndk, int a, int i, int m, int blk, int ms, R *__restrict__ HOSB,
                        const double *__restrict__ rcs, const double *__restrict__ rsn,
                        const SweepState *__restrict__ st)
{
    const int total = ndk * batch_items(mak, m);     // < 2^31 (checked on the host)
    const float rm = 1.0f / (float)m;
    for (int b = blockIdx.y; b < blk; b += gridDim.y) {
        if (st[b].done) continue;
        R *H = HOSB + (i64)b * ndk * mak * mak;
        const double *cs = rcs + (i64)b * ms, *sn = rsn + (i64)b * ms;
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
            const int u = e / ndk;
            batch_item<false, R>(H, ndk, mak, mak, a, i, m, cs, sn, u, e - u * ndk, rm);
        }
    }
}

// mode 0: initialise the sweep state from sumOffDiag; mode 1: end of a sweep.
__global__ void gpu_sweep_kernel(int mode, int nchunk, int bjmax, double bjtol,
                                 const double *__restrict__ partial, SweepState *__restrict__ st,
                                 int nblk)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    double s = 0.0;
    for (int i = 0; i < nchunk; ++i) s += partial[3 * ((i64)b * nchunk + i)];
    const double off = 2.0 * s;
    SweepState &S = st[b];
    if (mode == 0) {
        S.initye = off; S.ye = off; S.dye = off; S.k = 1; S.sumdiag = 0.0;
    } else {
        if (S.done) return;
        S.dye = off - S.ye;
        S.ye = S.ye + S.dye;
        S.k = S.k + 1;
    }
    S.done = !(fabs(S.dye) > S.initye * bjtol && S.k <= bjmax);
}

template <typename R>
__global__ void gpu_finish_kernel(int nchunk, int blk, int mak, int ndk, R *__restrict__ HOSB,
                                  double *__restrict__ EIG, const double *__restrict__ partial,
                                  SweepState *__restrict__ st, double *__restrict__ bstats)
{
    const int b = blockIdx.y;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < nchunk; ++i) s += partial[3 * ((i64)b * nchunk + i)];
        const SweepState &S = st[b];
        bstats[3 * (i64)b] = (double)S.k;
        bstats[3 * (i64)b + 1] = fabs(1.0 - S.ye / S.initye);
        bstats[3 * (i64)b + 2] = s;
    }
    R *H = HOSB + (i64)b * ndk * mak * mak;
    const i64 total = (i64)ndk * mak;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int kk = (int)(e % ndk), i = (int)(e / ndk);
        const i64 di = kk + (i64)ndk * (i + (i64)mak * i);
        EIG[kk + (i64)ndk * (i + (i64)mak * b)] = (double)H[di];
        H[di] = R(0);
    }
}

__global__ void identity_kernel(int mak, int blk, double *V)
{
    const i64 total = (i64)mak * mak * blk;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const i64 w = e % ((i64)mak * mak);
        V[e] = ((w % mak) == (w / mak)) ? 1.0 : 0.0;
    }
}

static int gridsz(i64 items)
{
    i64 g = (items + kThreads - 1) / kThreads;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (int)g;
}

// The spread schedule's sweeps of one level on stacked matrices H (element
// type R) in global memory: V, the sums and the angles in FP64.
template <typename R>
static int spread_sweeps(int bjmax, double bjtol, int blk, int mak, int ndk, R *H, double *VOSB, double *EIG,
                         double *d_bstats, cudaStream_t s)
{
    int rc = 0;
    const int gy = std::min(blk, 65535);
    const int npart_off = std::max(1, std::min(64, (int)(((i64)ndk * mak * mak + kThreads * 8 - 1) / (kThreads * 8))));
    const int ms = std::max(1, mak / 2);
    double *partial = nullptr, *rcs = nullptr;
    SweepState *st = nullptr;
    SC_CUDA(cudaMallocAsync(&partial, sizeof(double) * 3 * (size_t)npart_off * blk, s));
    SC_CUDA(cudaMallocAsync(&rcs, sizeof(double) * 2 * (size_t)ms * blk, s));
    SC_CUDA(cudaMallocAsync(&st, sizeof(SweepState) * (size_t)blk, s));
    double *rsn = rcs + (size_t)ms * blk;
    identity_kernel<<<gridsz((i64)mak * mak * blk), kThreads, 0, s>>>(mak, blk, VOSB);
    if (blk > 65535) { set_error("hosbdiag: %d blocks too many for the spread schedule", blk); rc = SCALIT_EINVAL; }
    if ((i64)ndk * mak * mak > 2147483647LL) { set_error("hosbdiag: a block of %d x %d x %d is too large", ndk, mak, mak); rc = SCALIT_EINVAL; }
    const dim3 goff(npart_off, blk);
    if (!rc) {
        gpu_partial_kernel<R><<<goff, kThreads, 0, s>>>(1, mak, ndk, H, partial);
        gpu_sweep_kernel<<<(blk + 127) / 128, 128, 0, s>>>(0, npart_off, bjmax, bjtol, partial, st, blk);
        SC_CHECK_LAUNCH();
    }
    std::vector<SweepState> hst(blk);
    const int max_ctas = 152 * 16;
    for (int sweep = 0; !rc && sweep <= bjmax + 1; ++sweep) {
        SC_CUDA(cudaMemcpyAsync(hst.data(), st, sizeof(SweepState) * blk, cudaMemcpyDeviceToHost, s));
        SC_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int b = 0; b < blk; ++b) any |= !hst[b].done;
        if (!any) break;
        for (int i = 1; i <= mak - 1; ++i) {
            for (int a = 0; a < mak - i; a += i) {
                const int m = std::min(i, mak - i - a);
                const i64 items = (i64)ndk * ((i64)(mak - 2 * m) * m + (i64)m * m);
                const int gx = (int)std::max<i64>(1, std::min<i64>((items + kThreads - 1) / kThreads,
                                                                   std::max(1, max_ctas / gy)));
                gpu_batch_angle_kernel<R><<<dim3(m, gy), kThreads, 0, s>>>(mak, ndk, a, i, blk, ms, H, rcs, rsn,
                                                                        VOSB, st);
                gpu_batch_rotate_kernel<R><<<dim3(gx, gy), kThreads, 0, s>>>(mak, ndk, a, i, m, blk, ms, H,
                                                                          rcs, rsn, st);
            }
        }
        SC_CHECK_LAUNCH();
        gpu_partial_kernel<R><<<goff, kThreads, 0, s>>>(1, mak, ndk, H, partial);
        gpu_sweep_kernel<<<(blk + 127) / 128, 128, 0, s>>>(1, npart_off, bjmax, bjtol, partial, st, blk);
        SC_CHECK_LAUNCH();
    }
    if (!rc) {
        const i64 items = (i64)ndk * mak;
        const int grot = (int)std::min<i64>((items + kThreads - 1) / kThreads, 152 * 8);
        gpu_partial_kernel<R><<<goff, kThreads, 0, s>>>(2, mak, ndk, H, partial);
        gpu_finish_kernel<R><<<dim3(grot, blk), kThreads, 0, s>>>(npart_off, blk, mak, ndk, H, EIG, partial, st, d_bstats);
        SC_CHECK_LAUNCH();
    }
    cudaFreeAsync(partial, s);
    cudaFreeAsync(rcs, s);
    cudaFreeAsync(st, s);
    return rc;
}

int hosbdiag_device(scalit_ctx *c, int bjmax, double bjtol, int blk, int mak, int ndk,
                    double *HOSB, double *VOSB, double *EIG, double *stats5, cudaStream_t s, bool f32)
{
    if (blk <= 0 || mak <= 0 || ndk <= 0) { set_error("hosbdiag: bad sizes"); return SCALIT_EINVAL; }
    std::vector<double> bstats(3 * (size_t)blk);
    double *d_bstats = nullptr;
    SC_CUDA(cudaMallocAsync(&d_bstats, sizeof(double) * 3 * (size_t)blk, s));
    int rc = 0;
    const size_t fixed = (96 + 5 * kMaxBatch) * sizeof(double);
    const size_t bytes = sizeof(double) * (size_t)ndk * mak * (ndk == 1 ? mak + 1 : mak);
    const bool per_block = (bytes + fixed <= 225 * 1024) && mak / 2 <= kMaxBatch;
    if (per_block) {
        SC_CUDA(cudaFuncSetAttribute(jacobi_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(225 * 1024)));
        const int grid = blk < 152 * 8 ? blk : 152 * 8;
        // threads: about 512 per SM shared by the CTAs that fit its shared
        // memory -- several blocks in flight hide the per-batch barriers and
        // angle latencies better than more warps in one.  Measured on GB300:
        // 96 x 96 blocks (two CTAs per SM) 0.36 s at 256 threads, 0.53 s at
        // 1024; 160 x 160 blocks (one) 5.39 s at 256, 4.76 s at 512, 4.89 s
        // at 1024.
        const int ctas = std::max(1, (int)((228 * 1024) / (fixed + bytes + 1024)));
        int nt = 256;
        while (nt < kJacThreads && 2 * nt * ctas <= 512) nt *= 2;
        static const int forced = [] {                 // SCALIT_JAC_THREADS: a tuning override
            const char *e = getenv("SCALIT_JAC_THREADS");
            const int v = e ? atoi(e) : 0;
            return (v >= 256 && v <= kJacThreads && v % 32 == 0) ? v : 0;   // above kMaxBatch
        }();
        if (forced) nt = forced;
        if (ndk == 1) {
            // one matrix per block: the packed triangle, half the shared memory
            // (a quarter with FP32 sweeps)
            const size_t pbytes = (f32 ? sizeof(float) : sizeof(double)) * (size_t)mak * (mak + 1) / 2;
            const int pctas = std::max(1, (int)((228 * 1024) / (fixed + pbytes + 1024)));
            int pnt = 256;
            while (pnt < 512 && 2 * pnt * pctas <= 512) pnt *= 2;
            if (forced) pnt = std::min(forced, 512);
            if (f32) {
                SC_CUDA(cudaFuncSetAttribute(jacobi_packed_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(225 * 1024)));
                jacobi_packed_kernel<float><<<grid, pnt, fixed + pbytes, s>>>(bjmax, bjtol, blk, mak, HOSB, VOSB,
                                                                              EIG, d_bstats);
            } else {
                SC_CUDA(cudaFuncSetAttribute(jacobi_packed_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(225 * 1024)));
                jacobi_packed_kernel<double><<<grid, pnt, fixed + pbytes, s>>>(bjmax, bjtol, blk, mak, HOSB, VOSB,
                                                                               EIG, d_bstats);
            }
        } else {
            jacobi_block_kernel<<<grid, nt, fixed + bytes, s>>>(bjmax, bjtol, blk, mak, ndk, HOSB, VOSB, EIG,
                                                                d_bstats);
        }
        SC_CHECK_LAUNCH();
    } else if (f32) {
        // FP32 sweeps on an FP32 copy of the stacks (the FP64 HOSB is left as
        // it came: the build reads only EIG0 and V after a level)
        float *Hf = nullptr;
        SC_CUDA(cudaMallocAsync(&Hf, sizeof(float) * (size_t)ndk * mak * mak * blk, s));
        rc = to_f32(HOSB, Hf, (i64)ndk * mak * mak * blk, s);
        if (!rc) rc = spread_sweeps<float>(bjmax, bjtol, blk, mak, ndk, Hf, VOSB, EIG, d_bstats, s);
        cudaFreeAsync(Hf, s);
        if (rc) { cudaFreeAsync(d_bstats, s); return rc; }
    } else {
        rc = spread_sweeps<double>(bjmax, bjtol, blk, mak, ndk, HOSB, VOSB, EIG, d_bstats, s);
        if (rc) { cudaFreeAsync(d_bstats, s); return rc; }
    }
    SC_CUDA(cudaMemcpyAsync(bstats.data(), d_bstats, sizeof(double) * 3 * (size_t)blk, cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    cudaFreeAsync(d_bstats, s);
    if (stats5) {
        double eff[5] = {INFINITY, -INFINITY, 0.0, 0.0, 0.0};
        for (int b = 0; b < blk; ++b) {
            const double k = bstats[3 * b], e0 = bstats[3 * b + 1], sd = bstats[3 * b + 2];
            eff[0] = std::min(eff[0], e0);
            eff[1] = std::max(eff[1], e0);
            eff[2] += e0; eff[3] += sd; eff[4] += k;
        }
        for (int i = 0; i < 5; ++i) stats5[i] = eff[i];
    }
    return rc;
}

// MJACOBI (src/iterate/libiterate/diag/jacobi.f90:2-83) as the external
// mjacobi_: one joint rotation of the (P, Q) plane (1-based) of all nin
// stacked nout x nout matrices HOUT(nin, nout, nout) on the device.  One CTA
// forms A = sum o^2, B = 2 sum o d, C = sum d^2 (o = HOUT(:, P, Q),
// d = (HOUT(:, P, P) - HOUT(:, Q, Q)) / 2) in a fixed order; the host takes the
// angle X from them with the reference's branches (atan of the host C
// library) and the rotation kernel updates the P and Q rows and columns with
// the reference's formulas.  *angle receives X, MJACOBI's result.
static constexpr int kMjT = 1024;
__global__ void __launch_bounds__(kMjT)
mjacobi_abc_kernel(int p, int q, int nout, int nin, const double *__restrict__ H, double *__restrict__ abc)
{
    const double *hpp = H + (i64)nin * (p + (i64)nout * p), *hqq = H + (i64)nin * (q + (i64)nout * q);
    const double *hpq = H + (i64)nin * (p + (i64)nout * q);
    double a = 0.0, b = 0.0, cc = 0.0;
    for (int k = threadIdx.x; k < nin; k += kMjT) {
        const double o = hpq[k], d = 0.5 * hpp[k] - 0.5 * hqq[k];
        a = fma(o, o, a);
        b = fma(o, d, b);
        cc = fma(d, d, cc);
    }
    __shared__ double red[3][kMjT / 32];
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        cc += __shfl_xor_sync(0xffffffffu, cc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = a;
        red[1][threadIdx.x >> 5] = b;
        red[2][threadIdx.x >> 5] = cc;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < kMjT / 32; ++w) t += red[threadIdx.x][w];
        abc[threadIdx.x] = (threadIdx.x == 1) ? 2.0 * t : t;
    }
}

__global__ void mjacobi_rotate_kernel(int p, int q, int nout, int nin, double cs, double sn, double *__restrict__ H)
{
    const double c2 = cs * cs, s2 = sn * sn, sc = sn * cs;
    const i64 total = (i64)nin * nout;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int k = (int)(e % nin), r = (int)(e / nin);
        if (r == p) {
            // the intersection block (p, p), (q, q), (p, q), (q, p)
            double *hpp = H + (i64)nin * (p + (i64)nout * p) + k, *hqq = H + (i64)nin * (q + (i64)nout * q) + k;
            double *hpq = H + (i64)nin * (p + (i64)nout * q) + k, *hqp = H + (i64)nin * (q + (i64)nout * p) + k;
            const double o = *hpq, d = 0.5 * *hpp - 0.5 * *hqq;
            const double np_ = c2 * *hpp + s2 * *hqq - 2 * sc * o;
            const double nq_ = c2 * *hqq + s2 * *hpp + 2 * sc * o;
            const double nqp = (c2 - s2) * o + 2 * sc * d;
            *hpp = np_;
            *hqq = nq_;
            *hpq = nqp;
            *hqp = nqp;
        } else if (r != q) {
            double *hrp = H + (i64)nin * (r + (i64)nout * p) + k, *hrq = H + (i64)nin * (r + (i64)nout * q) + k;
            double *hpr = H + (i64)nin * (p + (i64)nout * r) + k, *hqr = H + (i64)nin * (q + (i64)nout * r) + k;
            const double np_ = cs * *hrp - sn * *hrq;
            const double nq_ = cs * *hrq + sn * *hrp;
            *hrp = np_;
            *hpr = np_;
            *hrq = nq_;
            *hqr = nq_;
        }
    }
}

int mjacobi_device(int P, int Q, int nout, int nin, double *dH, double *dabc, double *angle, cudaStream_t s)
{
    const double PIE = 3.14159265358979323846264338328;
    const int p = P - 1, q = Q - 1;
    mjacobi_abc_kernel<<<1, kMjT, 0, s>>>(p, q, nout, nin, dH, dabc);
    SC_CHECK_LAUNCH();
    double abc[3];
    SC_CUDA(cudaMemcpyAsync(abc, dabc, sizeof(abc), cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    const double A = abc[0], B = abc[1], C = abc[2];
    double X;
    if (A == C) {
        X = (B == 0.0) ? 0.0 : -std::copysign(PIE / 8.0, B);
    } else {
        X = std::atan(B / (A - C)) / 4.0;
        if (A > C) X = (X < 0.0) ? X + PIE / 4.0 : X - PIE / 4.0;
    }
    const i64 total = (i64)nin * nout;
    const int grid = (int)std::max<i64>(1, std::min<i64>((total + 255) / 256, 152 * 8));
    mjacobi_rotate_kernel<<<grid, 256, 0, s>>>(p, q, nout, nin, std::cos(X), std::sin(X), dH);
    SC_CHECK_LAUNCH();
    *angle = X;
    return 0;
}

int osb_build(scalit_ctx *c, int bjmax, double bjtol, double *stats)
{
    const Layout &L = c->L;
    cudaStream_t s = c->stream;
    i64 hmax = 0;
    for (int l = 0; l < L.nlev; ++l) hmax = std::max(hmax, (i64)L.n[l] * L.N);
    double *HOSB = nullptr;
    SC_CUDA(cudaMallocAsync(&HOSB, sizeof(double) * (size_t)hmax, s));
    SC_CUDA(cudaMemcpyAsync(c->EIG0, c->RES, sizeof(double) * (size_t)L.N, cudaMemcpyDeviceToDevice, s));
    int rc = 0;
    for (int l = L.nlev - 1; l >= 0 && rc == 0; --l) {
        const auto t0 = std::chrono::steady_clock::now();
        const int mak = L.n[l];
        const i64 ndk = L.dim[l], blk = L.blk[l];
        if (ndk > 2147483647LL || blk > 2147483647LL) { set_error("level too large"); rc = SCALIT_EINVAL; break; }
        if (L.ndvr && l == L.nlev - 1) {
            rc = (cudaMemcpyAsync(HOSB, c->OUTH, sizeof(double) * (size_t)(mak * L.N), cudaMemcpyDeviceToDevice, s) == cudaSuccess) ? 0 : SCALIT_ECUDA;
        } else {
            const double *dep = L.dep[l] ? c->DEP + L.deps[l] : nullptr;
            hosb_init_kernel<<<gridsz((i64)mak * L.N), kThreads, 0, s>>>((int)blk, mak, (int)ndk, c->H0 + L.h0s[l], dep, c->EIG0, HOSB);
            if (cudaGetLastError() != cudaSuccess) { set_error("hosb init launch"); rc = SCALIT_ECUDA; }
        }
        if (rc == 0)
            rc = hosbdiag_device(c, bjmax, bjtol, (int)blk, mak, (int)ndk, HOSB, c->VOSB + L.vs[l],
                                 c->EIG0, stats ? stats + 5 * l : nullptr, s, c->build_prec == SCALIT_PREC_FP32);
        if (rc == 0 && cudaStreamSynchronize(s) != cudaSuccess) { set_error("osb build level %d", l + 1); rc = SCALIT_ECUDA; }
        c->build_s[l] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    cudaFreeAsync(HOSB, s);
    if (rc) return rc;
    rc = to_f32(c->EIG0, c->EIG0f, L.N, s);
    if (!rc) rc = to_f32(c->VOSB, c->VOSBf, L.vlen, s);
    if (!rc) { c->osb_built = true; osbw_invalidate(c); c->gen++; }
    SC_CUDA(cudaStreamSynchronize(s));
    if (!rc) rc = tc_prepare_px(c);
    if (!rc) rc = tc32_prepare(c, true);
    if (!rc) rc = px_half_prepare(c);
    return rc;
}

}  // namespace sc
