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
// rounding.  Two device schedules:
//  * many blocks (BLK >= 64): one CTA per block runs all its sweeps; the block
//    is staged in shared memory when it fits (level 1: n x n matrices);
//  * few blocks (the outermost levels, BLK = 1 for the angle): every rotation
//    is spread over the whole GPU -- one launch computes the partial A,B,C
//    sums, a second finishes the angle and rotates V, a third rotates HOSB.
// The angle is formed from A, B, C with square roots only (half-angle
// identities for atan(B/(A-C))/4 and the +-pi/4 shifts), which equals the
// reference's DATAN/DSIN/DCOS result to rounding.
#include "internal.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace sc {

static constexpr int kThreads = 256;

// cos and sin of the MJACOBI angle (jacobi.f90:42-60).
__device__ void jacobi_angle(double A, double B, double C, double *cs, double *sn)
{
    const double INV_SQRT2 = 0.70710678118654752440;
    if (A == C) {
        if (B == 0.0) { *cs = 1.0; *sn = 0.0; return; }
        // X = -sign(pi/8, B)
        const double c8 = sqrt(0.5 * (1.0 + INV_SQRT2));
        const double s8 = sqrt(0.5 * (1.0 - INV_SQRT2));
        *cs = c8;
        *sn = (B > 0.0) ? -s8 : s8;
        return;
    }
    const double T = B / (A - C);
    double c4, s4;   // cos, sin of atan(T)
    if (fabs(T) > 1.0) {
        const double r = 1.0 / T;
        const double h = sqrt(1.0 + r * r);
        c4 = fabs(r) / h;
        s4 = (T > 0.0 ? 1.0 : -1.0) / h;
    } else {
        c4 = 1.0 / sqrt(1.0 + T * T);
        s4 = T * c4;
    }
    const double c2 = sqrt(0.5 * (1.0 + c4));
    const double s2 = s4 / (2.0 * c2);
    double c = sqrt(0.5 * (1.0 + c2));
    double s = s2 / (2.0 * c);
    if (A > C) {
        double nc, ns;
        if (s < 0.0) {        // X + pi/4  (X < 0 <=> s < 0)
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

__device__ double block_offdiag(const double *H, int ndk, int mak, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    const i64 total = (i64)ndk * mak * mak;
    for (i64 e = threadIdx.x; e < total; e += blockDim.x) {
        const i64 rc = e / ndk;
        const int r = (int)(rc % mak), col = (int)(rc / mak);
        if (r < col) { const double h = H[e]; s = fma(h, h, s); }
    }
    block_sum3(s, z1, z2, red);
    return 2.0 * s;
}

__device__ double block_sumdiag(const double *H, int ndk, int mak, double *red)
{
    double s = 0.0, z1 = 0.0, z2 = 0.0;
    const i64 total = (i64)ndk * mak;
    for (i64 e = threadIdx.x; e < total; e += blockDim.x) {
        const int k = (int)(e % ndk), i = (int)(e / ndk);
        const double h = H[k + (i64)ndk * (i + (i64)mak * i)];
        s = fma(h, h, s);
    }
    block_sum3(s, z1, z2, red);
    return s;
}

// Rotate rows/columns p, q of every stacked matrix of one block (MJACOBI
// update, jacobi.f90:62-80) for the (k, r) items [e0, e1) in steps of `step`.
__device__ __forceinline__ void rotate_items(double *H, int ndk, int mak, int p, int q,
                                             double cs, double sn, i64 e0, i64 e1, i64 step)
{
    const double C2 = cs * cs, S2 = sn * sn, SC = sn * cs;
    for (i64 e = e0; e < e1; e += step) {
        const int k = (int)(e % ndk), r = (int)(e / ndk);
        if (r == q) continue;
        if (r == p) {
            double *hpp = H + k + (i64)ndk * (p + (i64)mak * p);
            double *hqq = H + k + (i64)ndk * (q + (i64)mak * q);
            double *hpq = H + k + (i64)ndk * (p + (i64)mak * q);
            double *hqp = H + k + (i64)ndk * (q + (i64)mak * p);
            const double odg = *hpq;
            const double ddg = 0.5 * *hpp - 0.5 * *hqq;
            const double np_ = C2 * *hpp + S2 * *hqq - 2 * SC * odg;
            const double nq_ = C2 * *hqq + S2 * *hpp + 2 * SC * odg;
            const double nqp = (C2 - S2) * odg + 2 * SC * ddg;
            *hpp = np_; *hqq = nq_; *hpq = nqp; *hqp = nqp;
        } else {
            double *hrp = H + k + (i64)ndk * (r + (i64)mak * p);
            double *hrq = H + k + (i64)ndk * (r + (i64)mak * q);
            double *hpr = H + k + (i64)ndk * (p + (i64)mak * r);
            double *hqr = H + k + (i64)ndk * (q + (i64)mak * r);
            const double a = *hrp, b = *hrq;
            const double np_ = cs * a - sn * b;
            const double nq_ = cs * b + sn * a;
            *hrp = np_; *hpr = np_; *hrq = nq_; *hqr = nq_;
        }
    }
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
__global__ void __launch_bounds__(kThreads)
jacobi_block_kernel(int bjmax, double bjtol, int blk, int mak, int ndk, int stage,
                    double *__restrict__ HOSB, double *__restrict__ VOSB, double *__restrict__ EIG,
                    double *__restrict__ bstats)
{
    extern __shared__ __align__(16) double smem[];
    double *red = smem;                 // 3 * 32
    double *rot = smem + 96;            // cs, sn
    double *Hs = smem + 128;            // staged block
    const int tid = threadIdx.x, nt = blockDim.x;
    const i64 bsz = (i64)ndk * mak * mak;
    for (int b = blockIdx.x; b < blk; b += gridDim.x) {
        double *Hg = HOSB + (i64)b * bsz;
        double *H = stage ? Hs : Hg;
        double *V = VOSB + (i64)b * mak * mak;
        __syncthreads();
        if (stage) for (i64 e = tid; e < bsz; e += nt) Hs[e] = Hg[e];
        for (i64 e = tid; e < (i64)mak * mak; e += nt) V[e] = ((e % mak) == (e / mak)) ? 1.0 : 0.0;
        __syncthreads();
        const double initye = block_offdiag(H, ndk, mak, red);
        double ye = initye, dye = initye;
        int k = 1;
        while (fabs(dye) > initye * bjtol && k <= bjmax) {
            for (int i = 1; i <= mak - 1; ++i) {
                for (int j = 1; j <= mak - i; ++j) {
                    const int p = j - 1, q = j + i - 1;
                    double sA = 0.0, sB = 0.0, sC = 0.0;
                    for (int kk = tid; kk < ndk; kk += nt) {
                        const double o = H[kk + (i64)ndk * (p + (i64)mak * q)];
                        const double d = 0.5 * H[kk + (i64)ndk * (p + (i64)mak * p)]
                                       - 0.5 * H[kk + (i64)ndk * (q + (i64)mak * q)];
                        sA = fma(o, o, sA); sB = fma(o, d, sB); sC = fma(d, d, sC);
                    }
                    if (ndk > 1) {
                        block_sum3(sA, sB, sC, red);
                    } else {
                        __syncthreads();
                        if (tid == 0) { red[0] = sA; red[1] = sB; red[2] = sC; }
                        __syncthreads();
                        sA = red[0]; sB = red[1]; sC = red[2];
                    }
                    if (tid == 0) {
                        double cs, sn;
                        jacobi_angle(sA, 2.0 * sB, sC, &cs, &sn);
                        rot[0] = cs; rot[1] = sn;
                    }
                    __syncthreads();
                    const double cs = rot[0], sn = rot[1];
                    rotate_items(H, ndk, mak, p, q, cs, sn, tid, (i64)ndk * mak, nt);
                    for (int a = tid; a < mak; a += nt) {
                        double *vp = V + (i64)p * mak, *vq = V + (i64)q * mak;
                        const double t = cs * vp[a] - sn * vq[a];
                        vq[a] = cs * vq[a] + sn * vp[a];
                        vp[a] = t;
                    }
                    __syncthreads();
                }
            }
            dye = block_offdiag(H, ndk, mak, red) - ye;
            ye = ye + dye;
            k = k + 1;
        }
        const double sd = block_sumdiag(H, ndk, mak, red);
        __syncthreads();
        for (i64 e = tid; e < (i64)ndk * mak; e += nt) {
            const int kk = (int)(e % ndk), i = (int)(e / ndk);
            const i64 di = kk + (i64)ndk * (i + (i64)mak * i);
            EIG[kk + (i64)ndk * (i + (i64)mak * b)] = H[di];
            H[di] = 0.0;
        }
        __syncthreads();
        if (stage) for (i64 e = tid; e < bsz; e += nt) Hg[e] = Hs[e];
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

static constexpr int kChunk = 8192;   // (k, r) items per CTA per rotation

__global__ void __launch_bounds__(kThreads)
gpu_partial_kernel(int mode, int mak, int ndk, int p, int q, const double *__restrict__ HOSB,
                   double *__restrict__ partial, const SweepState *__restrict__ st)
{
    // mode 0: A,B,C of plane (p,q); mode 1: sumOffDiag; mode 2: sumDiag.
    __shared__ double red[96];
    const int b = blockIdx.y;
    if (mode == 0 && st[b].done) return;
    const double *H = HOSB + (i64)b * ndk * mak * mak;
    double sA = 0.0, sB = 0.0, sC = 0.0;
    if (mode == 0) {
        const i64 k0 = (i64)blockIdx.x * kChunk;
        const i64 k1 = min((i64)ndk, k0 + kChunk);
        for (i64 kk = k0 + threadIdx.x; kk < k1; kk += blockDim.x) {
            const double o = H[kk + (i64)ndk * (p + (i64)mak * q)];
            const double d = 0.5 * H[kk + (i64)ndk * (p + (i64)mak * p)]
                           - 0.5 * H[kk + (i64)ndk * (q + (i64)mak * q)];
            sA = fma(o, o, sA); sB = fma(o, d, sB); sC = fma(d, d, sC);
        }
    } else if (mode == 1) {
        const i64 total = (i64)ndk * mak * mak;
        for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
            const i64 rc = e / ndk;
            const int r = (int)(rc % mak), col = (int)(rc / mak);
            if (r < col) { const double h = H[e]; sA = fma(h, h, sA); }
        }
    } else {
        const i64 total = (i64)ndk * mak;
        for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
            const int kk = (int)(e % ndk), i = (int)(e / ndk);
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

// One CTA per block: reduce the partials in order, form the angle, rotate V.
__global__ void gpu_angle_kernel(int nchunk, int mak, int p, int q, const double *__restrict__ partial,
                                 double *__restrict__ rot, double *__restrict__ VOSB,
                                 const SweepState *__restrict__ st)
{
    const int b = blockIdx.x;
    if (st[b].done) return;
    __shared__ double cssn[2];
    if (threadIdx.x == 0) {
        double A = 0.0, B = 0.0, C = 0.0;
        for (int i = 0; i < nchunk; ++i) {
            const double *pp = partial + 3 * ((i64)b * nchunk + i);
            A += pp[0]; B += pp[1]; C += pp[2];
        }
        double cs, sn;
        jacobi_angle(A, 2.0 * B, C, &cs, &sn);
        cssn[0] = cs; cssn[1] = sn;
        rot[2 * b] = cs; rot[2 * b + 1] = sn;
    }
    __syncthreads();
    const double cs = cssn[0], sn = cssn[1];
    double *V = VOSB + (i64)b * mak * mak;
    for (int a = threadIdx.x; a < mak; a += blockDim.x) {
        double *vp = V + (i64)p * mak, *vq = V + (i64)q * mak;
        const double t = cs * vp[a] - sn * vq[a];
        vq[a] = cs * vq[a] + sn * vp[a];
        vp[a] = t;
    }
}

__global__ void __launch_bounds__(kThreads)
gpu_rotate_kernel(int mak, int ndk, int p, int q, double *__restrict__ HOSB,
                  const double *__restrict__ rot, const SweepState *__restrict__ st)
{
    const int b = blockIdx.y;
    if (st[b].done) return;
    double *H = HOSB + (i64)b * ndk * mak * mak;
    const double cs = rot[2 * b], sn = rot[2 * b + 1];
    const i64 total = (i64)ndk * mak;
    rotate_items(H, ndk, mak, p, q, cs, sn, blockIdx.x * (i64)blockDim.x + threadIdx.x, total,
                 (i64)gridDim.x * blockDim.x);
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

__global__ void gpu_finish_kernel(int nchunk, int blk, int mak, int ndk, double *__restrict__ HOSB,
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
    double *H = HOSB + (i64)b * ndk * mak * mak;
    const i64 total = (i64)ndk * mak;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const int kk = (int)(e % ndk), i = (int)(e / ndk);
        const i64 di = kk + (i64)ndk * (i + (i64)mak * i);
        EIG[kk + (i64)ndk * (i + (i64)mak * b)] = H[di];
        H[di] = 0.0;
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

int hosbdiag_device(scalit_ctx *c, int bjmax, double bjtol, int blk, int mak, int ndk,
                    double *HOSB, double *VOSB, double *EIG, double *stats5, cudaStream_t s)
{
    if (blk <= 0 || mak <= 0 || ndk <= 0) { set_error("hosbdiag: bad sizes"); return SCALIT_EINVAL; }
    if (blk > 65535 && blk < 64) { set_error("hosbdiag: bad block count"); return SCALIT_EINVAL; }
    std::vector<double> bstats(3 * (size_t)blk);
    double *d_bstats = nullptr;
    SC_CUDA(cudaMallocAsync(&d_bstats, sizeof(double) * 3 * (size_t)blk, s));
    int rc = 0;
    const bool per_block = (blk >= 64) && ((i64)ndk * mak <= 262144);
    if (per_block) {
        const size_t bytes = sizeof(double) * (size_t)ndk * mak * mak;
        const size_t fixed = 128 * sizeof(double);
        const int stage = (bytes + fixed <= 225 * 1024) ? 1 : 0;
        const size_t smem = fixed + (stage ? bytes : 0);
        SC_CUDA(cudaFuncSetAttribute(jacobi_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(225 * 1024)));
        const int grid = blk < 152 * 8 ? blk : 152 * 8;
        jacobi_block_kernel<<<grid, kThreads, smem, s>>>(bjmax, bjtol, blk, mak, ndk, stage, HOSB,
                                                         VOSB, EIG, d_bstats);
        SC_CHECK_LAUNCH();
    } else {
        if (blk > 65535) { set_error("hosbdiag: %d blocks too many for the spread schedule", blk); cudaFreeAsync(d_bstats, s); return SCALIT_EINVAL; }
        const int nchunk = (int)((ndk + kChunk - 1) / kChunk);
        const int npart_off = std::max(1, std::min(64, (int)(((i64)ndk * mak * mak + kThreads * 8 - 1) / (kThreads * 8))));
        const int npart = std::max(nchunk, npart_off);
        double *partial = nullptr, *rot = nullptr;
        SweepState *st = nullptr;
        SC_CUDA(cudaMallocAsync(&partial, sizeof(double) * 3 * (size_t)npart * blk, s));
        SC_CUDA(cudaMallocAsync(&rot, sizeof(double) * 2 * (size_t)blk, s));
        SC_CUDA(cudaMallocAsync(&st, sizeof(SweepState) * (size_t)blk, s));
        identity_kernel<<<gridsz((i64)mak * mak * blk), kThreads, 0, s>>>(mak, blk, VOSB);
        const dim3 goff(npart_off, blk);
        gpu_partial_kernel<<<goff, kThreads, 0, s>>>(1, mak, ndk, 0, 0, HOSB, partial, st);
        gpu_sweep_kernel<<<(blk + 127) / 128, 128, 0, s>>>(0, npart_off, bjmax, bjtol, partial, st, blk);
        SC_CHECK_LAUNCH();
        std::vector<SweepState> hst(blk);
        const i64 items = (i64)ndk * mak;
        const int grot = (int)std::min<i64>((items + kThreads - 1) / kThreads, 152 * 8);
        for (int sweep = 0; sweep <= bjmax + 1; ++sweep) {
            SC_CUDA(cudaMemcpyAsync(hst.data(), st, sizeof(SweepState) * blk, cudaMemcpyDeviceToHost, s));
            SC_CUDA(cudaStreamSynchronize(s));
            bool any = false;
            for (int b = 0; b < blk; ++b) any |= !hst[b].done;
            if (!any) break;
            for (int i = 1; i <= mak - 1; ++i) {
                for (int j = 1; j <= mak - i; ++j) {
                    const int p = j - 1, q = j + i - 1;
                    gpu_partial_kernel<<<dim3(nchunk, blk), kThreads, 0, s>>>(0, mak, ndk, p, q, HOSB, partial, st);
                    gpu_angle_kernel<<<blk, 128, 0, s>>>(nchunk, mak, p, q, partial, rot, VOSB, st);
                    gpu_rotate_kernel<<<dim3(grot, blk), kThreads, 0, s>>>(mak, ndk, p, q, HOSB, rot, st);
                }
            }
            SC_CHECK_LAUNCH();
            gpu_partial_kernel<<<goff, kThreads, 0, s>>>(1, mak, ndk, 0, 0, HOSB, partial, st);
            gpu_sweep_kernel<<<(blk + 127) / 128, 128, 0, s>>>(1, npart_off, bjmax, bjtol, partial, st, blk);
            SC_CHECK_LAUNCH();
        }
        gpu_partial_kernel<<<goff, kThreads, 0, s>>>(2, mak, ndk, 0, 0, HOSB, partial, st);
        gpu_finish_kernel<<<dim3(grot, blk), kThreads, 0, s>>>(npart_off, blk, mak, ndk, HOSB, EIG, partial, st, d_bstats);
        SC_CHECK_LAUNCH();
        cudaFreeAsync(partial, s);
        cudaFreeAsync(rot, s);
        cudaFreeAsync(st, s);
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
                                 c->EIG0, stats ? stats + 5 * l : nullptr, s);
    }
    cudaFreeAsync(HOSB, s);
    if (rc) return rc;
    rc = to_f32(c->EIG0, c->EIG0f, L.N, s);
    if (!rc) rc = to_f32(c->VOSB, c->VOSBf, L.vlen, s);
    if (!rc) c->osb_built = true;
    SC_CUDA(cudaStreamSynchronize(s));
    return rc;
}

}  // namespace sc
