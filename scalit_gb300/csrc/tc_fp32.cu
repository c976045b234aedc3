// FP32 level contractions (the mixed-precision inner solves) on the tcgen05
// tensor cores in split-BF16 x3 form.
//
// Every FP32 operand value is split as x = hi + lo with hi = bf16(x) and
// lo = bf16(x - hi) (16 significant bits, relative error <= 2^-17), and
//   C = A_hi B_hi + A_hi B_lo + A_lo B_hi
// accumulates in one FP32 TMEM accumulator (the dropped lo*lo term is below
// 2^-16 of |A||B|).  Same operand mapping as the FP64 digit engine
// (tc_fp64.cu): A is the grid vector seen through the level's strides, B(k, n)
// = H(n, k) (pre-split once per level matrix, or per block for the
// preconditioner's rotations), C written with the level's epilogue (DEP row
// scale, the fused diagonal (V - shift) X, accumulation).
//
// A CTA (512 threads, 128 grid rows, one N tile of NT <= 256 columns) holds its
// whole B tile (all K steps, both halves) in shared memory; the FP32 operand
// streams through a cp.async ring of 16-wide K slabs, each cut into its hi/lo
// planes in the K-major canonical layout; thread 0 issues the three MMAs of a
// K step and commits them to the buffer's mbarrier, so cutting step k+1
// overlaps the MMAs of step k.  Every wait is bounded (error flag, drain,
// TMEM freed, return).
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace sc {

static constexpr int kBM32 = 128;
static constexpr int kThreads32 = 512;                      // cutting threads: four per grid row
static constexpr int kBlock32 = 544;                        // plus one warp that issues the MMAs
static constexpr int kStages32 = 6;
// Floats per slab stage: K-major rows (level 1) with a padded row stride of 20
// (16-byte aligned, conflict-free reads), M-major slabs 16 rows of 128 packed.
static constexpr int kSlab32 = kBM32 * 20;
static constexpr int kSlab32M = kBM32 * 16;
__host__ __device__ constexpr int slab_floats(bool kmajor) { return kmajor ? kSlab32 : kSlab32M; }
static constexpr int kAStep32 = 2 * kBM32 * 16 * 2;        // hi + lo planes of 128 x 16 BF16

struct Tc32Args {
    int M, N, K, KS, NT;
    i64 Mi, s1, s2, a_sk, c_sn;
    const float *A; i64 a_sz;
    float *C; i64 c_sz;
    const float *rowscale;
    int accumulate;
    float alpha;
    const float *diagV;
    const float *diagX;
    i64 dx_sz;
    float shift;
    const float *shiftv;
    const int *vgate;      // per-vector stop flags vgate[z * vgate_stride] (may be null)
    int vgate_stride;
    const int *gate;
    int *err;
    int vec;               // 16-byte operand loads (aligned rows / row groups, K % 4 == 0)
    int resident;          // every K slab of the grid operand in shared memory at once
    int cpre;              // accumulate: prefetch the output tile into the consumed slabs
    const uint4 *bsplit;   // [blocks][ntile][ks][hi, lo][NT x 16 BF16, canonical]
    int tpb;               // > 0: per-block B, tpb M tiles per block of Mi rows
    i64 b_blk;             // uint4 stride between blocks' planes
};

__global__ void __launch_bounds__(kBlock32, 2)
tc32_level_kernel(Tc32Args g)
{
    if (g.gate && *g.gate) return;
    if (g.vgate && g.vgate[(i64)blockIdx.z * g.vgate_stride]) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int NT = g.NT, KS = g.KS;
    const int bstep = 2 * NT * 32;                         // bytes of one K step of B (hi + lo)
    unsigned char *Bs = smem;                              // KS x bstep
    unsigned char *Abuf = Bs + (size_t)KS * bstep;         // 2 x kAStep32
    float *slabs = reinterpret_cast<float *>(Abuf + 2 * kAStep32);      // nslab x slab
    // resident: all KS slabs loaded at once; otherwise a ring of kStages32
    const bool resident = g.resident != 0;
    const int nslab = resident ? KS : kStages32;
    const int slab = slab_floats(g.a_sk == 1);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(slabs + nslab * slab);          // MMAs of a buffer done
    uint64_t *cutb = mbar + 2;                                                      // a buffer's planes cut
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 4);
    uint64_t *bready = mbar + 5;                                                    // the B tile landed

    const int tid = threadIdx.x, warp = tid >> 5;
    const int ntile = blockIdx.y, z = blockIdx.z;
    int m0, mlim;
    const uint4 *bsrc = g.bsplit;
    if (g.tpb > 0) {
        const int bsel = blockIdx.x / g.tpb, lt = blockIdx.x - bsel * g.tpb;
        m0 = bsel * (int)g.Mi + lt * kBM32;
        mlim = min(g.M, bsel * (int)g.Mi + (int)g.Mi);
        bsrc += (i64)bsel * g.b_blk;
    } else {
        m0 = blockIdx.x * kBM32;
        mlim = g.M;
    }
    const float *A = g.A + (i64)z * g.a_sz;
    float *C = g.C + (i64)z * g.c_sz;
    const uint32_t tcols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tslot)), "r"(tcols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init(&cutb[0], kThreads32);
        mbar_init(&cutb[1], kThreads32);
        mbar_init(bready, 1);
        mbar_init_fence();
        // the whole B tile (already split, canonical layout) by bulk copies,
        // one per K step, overlapping the grid operand's first loads
        const unsigned char *bsrc_b = reinterpret_cast<const unsigned char *>(bsrc + (i64)ntile * KS * (bstep / 16));
        mbar_arrive_expect_tx(bready, (uint32_t)(KS * bstep));
        for (int ks = 0; ks < KS; ++ks) bulk_g2s(Bs + (size_t)ks * bstep, bsrc_b + (size_t)ks * bstep, bstep, bready);
    }
    if (warp == kThreads32 / 32) {
        // the MMA warp: per K step wait for the cut planes, issue the three
        // MMAs (one lane), commit them to the buffer's barrier
        fence_before();
        __syncthreads();
        fence_after();
        const uint32_t tbase = *tslot;
        const uint32_t idesc = idesc_bf16(NT);
        const bool bok = mbar_wait(bready, 0);
        for (int ks = 0; ks < KS && bok; ++ks) {
            const int buf = ks & 1;
            if (!mbar_wait(&cutb[buf], (uint32_t)((ks >> 1) & 1))) break;
            fence_after();
            if ((tid & 31) == 0) {
                const unsigned char *Ab = Abuf + buf * kAStep32;
                const uint64_t a_hi = smem_desc(smem_addr(Ab), 128, 256);
                const uint64_t a_lo = smem_desc(smem_addr(Ab + kBM32 * 32), 128, 256);
                const unsigned char *Bk = Bs + (size_t)ks * bstep;
                const uint64_t b_hi = smem_desc(smem_addr(Bk), 128, 256);
                const uint64_t b_lo = smem_desc(smem_addr(Bk + NT * 32), 128, 256);
                tc_mma(tbase, a_hi, b_hi, idesc, ks > 0 ? 1u : 0u);
                tc_mma(tbase, a_hi, b_lo, idesc, 1u);
                tc_mma(tbase, a_lo, b_hi, idesc, 1u);
                tc_commit(&mbar[buf]);
            }
            __syncwarp();
        }
        fence_before();
        __syncthreads();
        return;   // warp 0 frees the TMEM
    }

    // row offsets with 32-bit quotients (M < 2^31)
    const int Mi32 = (int)g.Mi;
    auto row_off = [&](int mm) -> i64 {
        const int mq = mm / Mi32;
        return (i64)(mm - mq * Mi32) * g.s1 + (i64)mq * g.s2;
    };
    const int row = tid & (kBM32 - 1), q = tid >> 7;
    const int m = m0 + row;
    const bool mvalid = m < mlim;
    const i64 moff = mvalid ? row_off(m) : 0;
    const bool rowc = (g.a_sk == 1);
    i64 lmoff[4];
    bool lvalid[4];
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = rowc ? ((tid >> 4) + 32 * i) : row;
        const int mm = m0 + r;
        lvalid[i] = mm < mlim;
        lmoff[i] = (lvalid[i] && !g.vec) ? row_off(mm) : 0;
    }
    // 16-byte loads: K-major rows take four consecutive k per thread, M-major
    // slabs four consecutive rows (one block: Mi % 4 == 0) at one k
    const int vr = rowc ? (tid >> 2) : 4 * (tid & 31);
    const int vj = rowc ? 4 * (tid & 3) : (tid >> 5);
    bool vvalid = false;
    i64 vmoff = 0;
    if (g.vec) {
        const int mm = m0 + vr;
        vvalid = mm < mlim;
        vmoff = vvalid ? row_off(mm) : 0;
    }
    auto issue = [&](int t) {
        if (t < KS && g.vec) {
            float *st = slabs + (resident ? t : t % kStages32) * slab;
            const int k = t * 16 + vj;
            float *dst = rowc ? st + vr * 20 + vj : st + vj * kBM32 + vr;
            if (vvalid && k < g.K) {
                const float *src = A + vmoff + (i64)k * g.a_sk;
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(smem_addr(dst)), "l"(src) : "memory");
            } else {
                *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else if (t < KS) {
            float *st = slabs + (resident ? t : t % kStages32) * slab;
            #pragma unroll
            for (int i = 0; i < 4; ++i) {
                int r, j;
                if (rowc) { j = tid & 15; r = (tid >> 4) + 32 * i; }
                else { r = row; j = q + 4 * i; }
                const int k = t * 16 + j;
                float *dst = rowc ? st + r * 20 + j : st + j * kBM32 + r;
                if (lvalid[i] && k < g.K) {
                    const float *src = A + lmoff[i] + (i64)k * g.a_sk;
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(smem_addr(dst)), "l"(src) : "memory");
                } else {
                    *dst = 0.0f;
                }
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // resident: every slab in flight at once; otherwise a ring with
    // kStages32 - 1 slabs of look-ahead
    if (resident) {
        for (int t = 0; t < KS; ++t) issue(t);
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else {
        for (int t = 0; t < kStages32 - 1; ++t) issue(t);
    }

    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *tslot;
    bool ok = true;
    for (int ks = 0; ks < KS; ++ks) {
        const int buf = ks & 1;
        if (ks >= 2 && !mbar_wait(&mbar[buf], ((ks - 2) >> 1) & 1)) { ok = false; break; }
        if (!resident) {
            asm volatile("cp.async.wait_group %0;" :: "n"(kStages32 - 2) : "memory");
            asm volatile("bar.sync 1, %0;" :: "n"(kThreads32) : "memory");   // cutting threads only
            issue(ks + kStages32 - 1);
        }
        const float *st = slabs + (resident ? ks : ks % kStages32) * slab;
        unsigned char *Ab = Abuf + buf * kAStep32;
        uint32_t hw[2], lw[2];
        #pragma unroll
        for (int jj = 0; jj < 4; jj += 2) {
            const int j0 = q * 4 + jj;
            const float x0 = rowc ? st[row * 20 + j0] : st[j0 * kBM32 + row];
            const float x1 = rowc ? st[row * 20 + j0 + 1] : st[(j0 + 1) * kBM32 + row];
            const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
            const __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
            const __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
            hw[jj >> 1] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
            lw[jj >> 1] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        const int rowoff = (row >> 3) * 256 + (q >> 1) * 128 + (row & 7) * 16 + (q & 1) * 8;
        *reinterpret_cast<uint2 *>(Ab + rowoff) = make_uint2(hw[0], hw[1]);
        *reinterpret_cast<uint2 *>(Ab + kBM32 * 32 + rowoff) = make_uint2(lw[0], lw[1]);
        // make the planes (and the preloaded B tile) visible to the tensor cores
        fence_proxy_async_smem();
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_addr(&cutb[buf])) : "memory");
    }
    // accumulating, resident, M-major output: once every slab is converted
    // (a barrier of the cutting threads; the resident loop has none), the
    // tile of C to add to streams into the consumed slabs while the last MMAs
    // finish, so the epilogue reads it from shared memory
    const float *Cs = slabs;                                  // [NT][kBM32]
    if (g.cpre) {
        asm volatile("bar.sync 1, %0;" :: "n"(kThreads32) : "memory");
        const int rg = 4 * (tid & 31);
        if (m0 + rg < mlim) {
            const float *csrc = C + row_off(m0 + rg);
            for (int n = tid >> 5; n < NT && ntile * NT + n < g.N; n += kThreads32 / 32)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                             :: "r"(smem_addr(Cs + n * kBM32 + rg)), "l"(csrc + (i64)(ntile * NT + n) * g.c_sn)
                             : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    if (ok) ok = mbar_wait(&mbar[(KS - 1) & 1], ((KS - 1) >> 1) & 1);
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (g.cpre) asm volatile("bar.sync 1, %0;" :: "n"(kThreads32) : "memory");
    if (!ok) {
        if (g.err) atomicExch(g.err, 3);
        for (int b = 0; b < 2; ++b) mbar_wait(&mbar[b], 0) || mbar_wait(&mbar[b], 1);
    }
    fence_after();
    if (g.c_sn == 1) {
        // Output rows contiguous along n (a level with nin == 1): a thread owns
        // one row, so storing straight from TMEM would give every warp store 32
        // rows a row length apart.  The scaled accumulator tile goes through
        // shared memory instead (the B tile and A planes, free once the last
        // MMA completed; padded stride NT + 1), and each warp then finishes
        // whole rows with the lanes along n: the diagonal term's loads, the
        // accumulated output and the stores are all coalesced.
        float *stage = reinterpret_cast<float *>(smem);
        const int ld = NT + 1;
        const float rs = (g.rowscale && mvalid) ? g.rowscale[m % g.Mi] : 1.0f;
        const float sc = g.alpha * rs;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int cq = NT / 4;
        const int cbeg = (warp >> 2) * cq, cend = cbeg + cq;
        for (int c0 = cbeg; c0 < cend && ok; c0 += 4) {
            float v[4];
            tmem_ld4(tbase + lane_base + (uint32_t)c0, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            #pragma unroll
            for (int j = 0; j < 4; ++j) stage[row * ld + c0 + j] = sc * v[j];
        }
        // every cutting thread arrives here, whatever its wait results were
        asm volatile("bar.sync 1, %0;" :: "n"(kThreads32) : "memory");
        const float shift = g.shiftv ? g.shiftv[z] : g.shift;
        const int lane = tid & 31;
        for (int r = warp; r < kBM32 && ok; r += kThreads32 / 32) {
            if (m0 + r >= mlim) break;
            const i64 ro = row_off(m0 + r);
            for (int cc = lane; cc < NT; cc += 32) {
                const int n = ntile * NT + cc;
                if (n >= g.N) break;
                const i64 p = ro + n;
                float out = stage[r * ld + cc];
                if (g.diagV) out = fmaf(g.alpha * (g.diagV[p] - shift), g.diagX[p + (i64)z * g.dx_sz], out);
                if (g.accumulate) out += C[p];
                C[p] = out;
            }
        }
    } else if (ok) {
        // warp w reads TMEM lanes 32 (w % 4) .. (its rows) and the column quarter w / 4
        const float rs = (g.rowscale && mvalid) ? g.rowscale[m % g.Mi] : 1.0f;
        const float sc = g.alpha * rs;
        const float shift = g.shiftv ? g.shiftv[z] : g.shift;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int cq = NT / 4;
        const int cbeg = (warp >> 2) * cq, cend = cbeg + cq;
        // 8 columns at a time: two TMEM loads, one wait, then every global
        // load of the group (diagonal, accumulated output) before any store
        for (int c0 = cbeg; c0 < cend; c0 += 8) {
            float v[2][4];
            #pragma unroll
            for (int q = 0; q < 2; ++q)
                if (c0 + 4 * q < cend) tmem_ld4(tbase + lane_base + (uint32_t)(c0 + 4 * q), v[q]);   // warp-uniform
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!mvalid) continue;
            float outv[2][4];
            #pragma unroll
            for (int q = 0; q < 2; ++q)
                #pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int n = ntile * NT + c0 + 4 * q + j;
                    if (c0 + 4 * q >= cend || n >= g.N) continue;
                    const i64 p = moff + (i64)n * g.c_sn;
                    float out = sc * v[q][j];
                    if (g.diagV) out = fmaf(g.alpha * (g.diagV[p] - shift), g.diagX[p + (i64)z * g.dx_sz], out);
                    if (g.accumulate) out += g.cpre ? Cs[(c0 + 4 * q + j) * kBM32 + row] : C[p];
                    outv[q][j] = out;
                }
            #pragma unroll
            for (int q = 0; q < 2; ++q)
                #pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int n = ntile * NT + c0 + 4 * q + j;
                    if (c0 + 4 * q < cend && n < g.N) C[moff + (i64)n * g.c_sn] = outv[q][j];
                }
        }
    }
    // the B copies have landed before the CTA's shared memory goes (they
    // have on every path that issued an MMA; this covers an early stop)
    if (tid == 0) mbar_wait(bready, 0);
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(tcols) : "memory");
}

// hi/lo planes of B(k, n) = H(n, k) for blk matrices H (n x n, column-major,
// consecutive), H = M_b (transpose = 0) or M_b^T (1), in the canonical layout
// [block][tile][ks][hi, lo][NT x 16].
__global__ void split_b_kernel(int nout, int NT, int ntiles, int KS, int blk, const float *__restrict__ Mt,
                               int transpose, uint16_t *__restrict__ out)
{
    const i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    const i64 total = (i64)blk * nout * nout;
    if (idx >= total) return;
    const int b = (int)(idx / ((i64)nout * nout));
    const int rem = (int)(idx - (i64)b * nout * nout);
    const int n = rem % nout, k = rem / nout;
    const float *Mb = Mt + (i64)b * nout * nout;
    const float x = transpose ? Mb[k + (i64)n * nout] : Mb[n + (i64)k * nout];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    const int tile = n / NT, nn = n % NT, ks = k / 16, kk = k % 16;
    const size_t base = ((((size_t)b * ntiles + tile) * KS + ks) * 2) * (size_t)NT * 16;
    const size_t off = (size_t)(nn >> 3) * 128 + (size_t)(kk >> 3) * 64 + (size_t)(nn & 7) * 8 + (kk & 7);
    out[base + off] = __bfloat16_as_ushort(h);
    out[base + (size_t)NT * 16 + off] = __bfloat16_as_ushort(l);
}

// One N tile holds every output column up to 176 (the grid operand is then
// loaded and split once; B, the ring and the A buffers fit one CTA's shared
// memory); wider levels take two tiles.
static void plan_dims(int nout, int &NT, int &ntiles, int &KS)
{
    const int n16 = (nout + 15) / 16 * 16;
    NT = n16 <= 176 ? n16 : ((nout + 1) / 2 + 15) / 16 * 16;
    ntiles = (nout + NT - 1) / NT;
    KS = (nout + 15) / 16;
}

// 16-byte loads of the grid operand: K-major rows (a_sk == 1) need K and the
// row stride a multiple of 4; M-major slabs need blocks of a multiple of 4
// rows and 4-aligned strides; both a 16-byte aligned base and vector stride.
static int vec_ok(const Tc32Args &g)
{
    if ((reinterpret_cast<uintptr_t>(g.A) & 15) || (g.a_sz % 4)) return 0;
    if (g.a_sk == 1) return (g.K % 4 == 0 && g.s1 % 4 == 0 && g.s2 % 4 == 0) ? 1 : 0;
    return (g.s1 == 1 && g.Mi % 4 == 0 && g.s2 % 4 == 0 && g.a_sk % 4 == 0) ? 1 : 0;
}

static int split_into(scalit_ctx *c, TcLevelData &t, int nout, int blk, const float *Mt, int transpose)
{
    int NT, ntiles, KS;
    plan_dims(nout, NT, ntiles, KS);
    const size_t nel = (size_t)blk * ntiles * KS * 2 * NT * 16;
    SC_CUDA(cudaMalloc(&t.dig, nel * sizeof(uint16_t)));
    SC_CUDA(cudaMemsetAsync(t.dig, 0, nel * sizeof(uint16_t), c->stream));
    const i64 items = (i64)blk * nout * nout;
    split_b_kernel<<<(int)((items + 255) / 256), 256, 0, c->stream>>>(nout, NT, ntiles, KS, blk, Mt, transpose,
                                                                      t.dig);
    SC_CHECK_LAUNCH();
    t.NT = NT; t.ntiles = ntiles; t.KS = KS; t.usable = 1;
    return 0;
}

void tc32_free(scalit_ctx *c, bool levels, bool rotations)
{
    for (int l = 0; l < SCALIT_FMAX; ++l) {
        if (levels && c->tc32[l].dig) { cudaFree(c->tc32[l].dig); c->tc32[l] = TcLevelData{}; }
        for (int d = 0; d < 2 && rotations; ++d)
            if (c->pxtc32[l][d].dig) { cudaFree(c->pxtc32[l][d].dig); c->pxtc32[l][d] = TcLevelData{}; }
    }
}

// Level matrices (after load) and, when the preconditioner exists, its rotations.
int tc32_prepare(scalit_ctx *c, bool rotations)
{
    const Layout &L = c->L;
    tc32_free(c, !rotations, rotations);
    if (!rotations) {
        for (int l = 0; l < L.nlev; ++l) {
            if (L.ndvr && l == L.nlev - 1) continue;
            if (L.n[l] > 256) continue;
            int rc = split_into(c, c->tc32[l], L.n[l], 1, c->H0f + L.h0s[l], 0);
            if (rc) return rc;
        }
    } else {
        for (int l = 1; l < L.nlev; ++l) {
            if (L.n[l] > 256 || L.dim[l] < 2) continue;
            for (int d = 0; d < 2; ++d) {
                int rc = split_into(c, c->pxtc32[l][d], L.n[l], (int)L.blk[l], c->VOSBf + L.vs[l], d);
                if (rc) return rc;
            }
        }
    }
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

static size_t smem_bytes(int NT, int KS, int nslab, int slab)
{
    return (size_t)KS * 2 * NT * 32 + 2 * (size_t)kAStep32 + (size_t)nslab * slab * 4 + 96;
}

static int launch32(const Tc32Args &g, i64 gx, int ntiles, int nvec, cudaStream_t s)
{
    // all K slabs resident when they fit (every load in flight at once), else the ring
    const int slab = slab_floats(g.a_sk == 1);
    const int resident = (g.KS <= kStages32 || smem_bytes(g.NT, g.KS, g.KS, slab) <= 220 * 1024) ? 1 : 0;
    const size_t smem = smem_bytes(g.NT, g.KS, resident ? g.KS : kStages32, slab);
    if (smem > 220 * 1024) { set_error("tensor-core FP32 tile too large"); return SCALIT_EUNSUP; }
    // the staged epilogue of row-contiguous outputs reuses the B tile and A planes
    if (g.c_sn == 1 && (size_t)kBM32 * (g.NT + 1) * 4 > (size_t)g.KS * 2 * g.NT * 32 + 2 * (size_t)kAStep32) {
        set_error("tensor-core FP32 output stage does not fit");
        return SCALIT_EUNSUP;
    }
    static int configured = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaFuncSetAttribute(tc32_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        configured = dev;
    }
    if (gx > 2147483647LL || nvec > 65535) { set_error("tensor-core FP32 grid too large"); return SCALIT_EINVAL; }
    Tc32Args gv = g;
    gv.vec = vec_ok(g);
    gv.resident = resident;
    // output prefetch: 16-byte groups of four rows of one block at one column
    gv.cpre = (resident && g.accumulate && g.s1 == 1 && g.Mi % 4 == 0 && g.s2 % 4 == 0 && g.c_sn % 4 == 0 &&
               g.c_sz % 4 == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0 &&
               (size_t)g.NT * kBM32 <= (size_t)g.KS * slab_floats(false)) ? 1 : 0;
    tc32_level_kernel<<<dim3((unsigned)gx, ntiles, nvec), kBlock32, smem, s>>>(gv);
    SC_CHECK_LAUNCH();
    return 0;
}

bool tc32_usable(const scalit_ctx *c, int l)
{
    return c->fp32_mode == SCALIT_FP32_TENSOR && c->tc32[l].usable;
}

bool tc32_px_usable(const scalit_ctx *c, int l)
{
    return (c->fp32_mode == SCALIT_FP32_TENSOR || c->fp32_mode == SCALIT_FP32_TENSOR_PX ||
            c->fp32_mode == SCALIT_FP32_TENSOR16) &&
           c->pxtc32[l][0].usable && c->pxtc32[l][1].usable;
}

int tc32_level_apply(const scalit_ctx *c, int l, const float *X, float *Y, int accumulate, const float *diagV,
                     float shift, float alpha, const int *gate, cudaStream_t s, int nvec, const float *shiftv,
                     const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const TcLevelData &t = c->tc32[l];
    if (!t.usable) { set_error("level %d has no FP32 tensor-core plan", l + 1); return SCALIT_EUNSUP; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    Tc32Args g{};
    g.N = nout; g.K = nout; g.KS = t.KS; g.NT = t.NT;
    if (nin == 1) {
        g.M = (int)blk; g.Mi = blk; g.s1 = nout; g.s2 = 0; g.a_sk = 1; g.c_sn = 1;
        g.rowscale = nullptr;
    } else {
        const i64 M = nin * blk;
        if (M > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
        g.M = (int)M; g.Mi = nin; g.s1 = 1; g.s2 = nin * nout; g.a_sk = nin; g.c_sn = nin;
        g.rowscale = L.dep[l] ? c->DEPf + L.deps[l] : nullptr;
    }
    g.A = X; g.a_sz = N; g.C = Y; g.c_sz = N;
    g.accumulate = accumulate; g.alpha = alpha;
    g.diagV = diagV; g.diagX = X; g.dx_sz = N; g.shift = shift; g.shiftv = shiftv;
    g.vgate = vgate; g.vgate_stride = vstride;
    g.gate = gate; g.err = c->tc_err;
    g.bsplit = reinterpret_cast<const uint4 *>(t.dig);
    return launch32(g, (g.M + kBM32 - 1) / kBM32, t.ntiles, nvec, s);
}

int tc32_rot_apply(const scalit_ctx *c, int l, int transpose, const float *X, float *Y, const int *gate,
                   cudaStream_t s, int nvec, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const TcLevelData &t = c->pxtc32[l][transpose ? 1 : 0];
    if (!t.usable) { set_error("level %d has no FP32 tensor-core rotation plan", l + 1); return SCALIT_EUNSUP; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    const i64 M = nin * blk;
    if (M > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
    Tc32Args g{};
    g.N = nout; g.K = nout; g.KS = t.KS; g.NT = t.NT;
    g.M = (int)M; g.Mi = nin; g.s1 = 1; g.s2 = nin * nout; g.a_sk = nin; g.c_sn = nin;
    g.A = X; g.a_sz = N; g.C = Y; g.c_sz = N;
    g.alpha = 1.0f; g.gate = gate; g.err = c->tc_err;
    g.vgate = vgate; g.vgate_stride = vstride;
    g.bsplit = reinterpret_cast<const uint4 *>(t.dig);
    i64 gx;
    if (blk > 1) {
        g.tpb = (int)((nin + kBM32 - 1) / kBM32);
        g.b_blk = (i64)t.ntiles * t.KS * 2 * t.NT * 2;     // uint4 per block
        gx = blk * g.tpb;
    } else {
        gx = (M + kBM32 - 1) / kBM32;
    }
    return launch32(g, gx, t.ntiles, nvec, s);
}

}  // namespace sc
