// Persistent FP32 level products of H*X on the tcgen05 tensor cores.
//
// One CTA per SM walks a strided sequence of 128-row tiles of the grid
// operand (all vectors of the launch), with the level matrix held in shared
// memory for the whole launch.  Four roles run a pipeline:
//
//   load lane (warp 17)     requests 16-wide K slabs of the FP32 grid operand
//                           by TMA tensor copies into a ring of shared-memory
//                           slots (6-7 deep; slot "full" and "empty"
//                           mbarriers);
//   MMA lane (warp 16)      issues the three products of every K step into one
//                           of two TMEM accumulators, committing them to the
//                           plane's "free" barrier and, after a tile's last K
//                           step, to the accumulator's "full" barrier;
//   converters (warps 0-7)  cut each landed slab into its hi/lo planes
//                           (K-major canonical layout) in a second ring, two K
//                           steps per pass, and release the slot;
//   epilogue (warps 8-15)   drain a full accumulator (scales, DEP row factor,
//                           fused diagonal term, accumulation) while the next
//                           tile's products run in the other accumulator.
//
// Split forms, both accumulated in FP32 TMEM:
//   FP16 (default): every vector is scaled by 2^e_x so that max|x| lies in
//     [2^14, 2^15), every output column of B by 2^e_n likewise; each scaled
//     value v is cut as hi = f16(v), lo = f16(v - hi) (22 significant bits) and
//     C = (A_hi B_hi + A_hi B_lo + A_lo B_hi) 2^-(e_x + e_n).  The dropped
//     lo*lo term and the cut leave ~2^-21 relative error of |A||B|, the
//     accuracy class of an FP32 CUDA-core GEMM of the same K.  e_x comes from
//     a max-reduction of each vector (absmax_bits_kernel) before the levels.
//   BF16: hi = bf16(x), lo = bf16(x - hi) without scaling (16 bits).
//
// Operand mapping (as in tc_fp32.cu): A(m, k) is the grid vector seen
// through the level's strides, B(k, n) = H(n, k), C written with the level's
// epilogue.  Rows contiguous along k (level 1): the slab is one 2-D box
// (16 k x 128 rows, 64-byte swizzle) of the view [vector][row][k]; the
// outputs, contiguous along n, leave through a 32 x 16 stage per epilogue
// warp, stored by TMA in the same swizzle.  Otherwise (the grid point index
// fastest within blocks of Mi points, Mi % 32 == 0) a tile's 128 rows are
// four groups of 32 points; the groups of one block form a run, moved as one
// box of 32 points x w groups x 16 k of the view
// [vector][block][k][group][point] (one box per tile when the blocks hold
// whole tiles, two when a tile straddles a block boundary: each TMA
// instruction costs its issuing thread about 0.2 us, so fewer and larger
// boxes keep the load lanes ahead), and a warp's 32 TMEM lanes are 32
// consecutive grid points of one output column.  The epilogue writes its
// results over the accumulated output's place in the ring; once the four
// quarters of a chunk are written, one lane stores the chunk's runs.
//
// Every mbarrier wait is bounded; an expired wait raises a shared abort flag
// after which no role waits again, the load and MMA lanes stop issuing and
// let the copies and products in flight complete, the error word is set and
// the CTA frees its TMEM and returns.
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace sc {

static constexpr int kPM = 128;                       // grid rows per tile = TMEM lanes
static constexpr int kPConv = 256;                    // converter threads
static constexpr int kPEpiWarps = 8;                  // two per TMEM lane quarter
static constexpr int kPThreads = kPConv + 32 * kPEpiWarps + 96;
static constexpr int kPMmaWarp = kPConv / 32 + kPEpiWarps;     // the MMA lane
static constexpr int kPLoadWarp = kPMmaWarp + 1;               // the TMA load lane
static constexpr int kPELoadWarp = kPMmaWarp + 2;              // the epilogue operands' load lane
static constexpr int kPERingMax = 8;                           // epilogue operand chunks in flight
static constexpr int kPSlotsMax = 7;                  // FP32 slab slots (rows along k: 7; else 6)
static constexpr int kPSlotsM = 6;
static constexpr int kPPlanes = 4;                    // hi/lo plane slots
static constexpr int kPSlab = kPM * 16 * 4;           // one FP32 slab: 8 KB
static constexpr int kPPlane = kPM * 16 * 2 * 2;      // hi + lo planes: 8 KB
static constexpr int kPStage = 32 * 16;               // floats per epilogue stage (2 per warp)
static constexpr int kPAccCols = 256;                 // TMEM columns per accumulator
static constexpr int kPMaxSmem = 227 * 1024;
static constexpr int kPMaxVec = 4096;                 // vectors per launch (scale slots)

struct Tc32pArgs {
    int M, K, KS, NT, N;       // rows per vector, contraction, K steps, tile columns, output columns
    int mtiles, tiles;         // M tiles per vector, M tiles x vectors
    i64 Mi, s1, s2, a_sk, c_sn;
    float *C; i64 c_sz;
    const float *rowscale;
    int accumulate;
    float alpha;
    const float *diagV;
    const float *diagX; i64 dx_sz;
    float shift;
    const float *shiftv;
    const int *vgate; int vgate_stride;
    const int *gate;
    int *err;
    const uint4 *bsplit;       // [KS][hi, lo][NT x 16] canonical K-major
    const float *binv;         // per output column: 2^-e_n (FP16 form)
    const unsigned *xmax;      // per vector: bits of max |x| (FP16 form)
    int tstore;                // outputs contiguous along n, nothing to add: TMA stores
    int ering, echunk;         // points fastest: epilogue operand ring slots and bytes per slot
    int nslots;                // FP32 slab slots
    int gp, nblk;              // points fastest: groups of 32 points per block, blocks per vector
};

// Tensor maps of one launch.  Rows along k: a[0] (the grid operand) and c[0]
// (level-1 output stores).  Points fastest: entry w - 1 holds boxes of
// 32 points x w groups of 32 points x 16 k (or n), w = 1..4, for the grid
// operand (a), the output (c) and V (v).
struct Tc32pMaps {
    CUtensorMap a[4], c[4], v[4];
};

// Shared memory: B, slab slots, plane slots, the epilogue region (level 1:
// two 32 x 16 stages per epilogue warp; otherwise the operand ring), column
// scales, barriers.
static size_t p_fixed_bytes(int NT, int KS, int nslots)
{
    return (size_t)KS * 2 * NT * 32 + (size_t)nslots * kPSlab + (size_t)kPPlanes * kPPlane + 256 * 4 +
           (2 * kPSlotsMax + 2 * kPPlanes + 3 * kPERingMax + 6) * 8 + 16;
}
static constexpr size_t kPStageBytes = (size_t)kPEpiWarps * 2 * kPStage * 4;

static size_t p_smem_bytes(int NT, int KS, int nslots, size_t ebytes)
{
    return p_fixed_bytes(NT, KS, nslots) + (ebytes > kPStageBytes ? ebytes : kPStageBytes);
}

// Scale exponent e with max|v| 2^e in [2^14, 2^15) from the bits of max|v|
// (clamped so 2^e and 2^-e stay normal; inf/NaN give a tiny scale and stay
// non-finite).
__host__ __device__ __forceinline__ int p_scale_exp(unsigned bits)
{
    const int ef = (int)((bits >> 23) & 0xFFu);
    int e = 141 - ef;
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    return e;
}

__device__ __forceinline__ float p_pow2(int e) { return __int_as_float((e + 127) << 23); }

// Two values at once: hi/lo halves packed as the MMA reads them (lower k in
// the low 16 bits).
template <bool F16>
__device__ __forceinline__ void p_cut2(float x0, float x1, float xs, uint32_t &hw, uint32_t &lw)
{
    if constexpr (F16) {
        const float2 v = make_float2(x0 * xs, x1 * xs);
        const __half2 hh = __float22half2_rn(v);
        const float2 hb = __half22float2(hh);
        const __half2 ll = __float22half2_rn(make_float2(v.x - hb.x, v.y - hb.y));
        hw = *reinterpret_cast<const uint32_t *>(&hh);
        lw = *reinterpret_cast<const uint32_t *>(&ll);
    } else {
        const __nv_bfloat162 hh = __float22bfloat162_rn(make_float2(x0, x1));
        const float2 hb = __bfloat1622float2(hh);
        const __nv_bfloat162 ll = __float22bfloat162_rn(make_float2(x0 - hb.x, x1 - hb.y));
        hw = *reinterpret_cast<const uint32_t *>(&hh);
        lw = *reinterpret_cast<const uint32_t *>(&ll);
    }
}

// Points fastest: a tile's 128 rows are the groups of 32 points G0 .. G0 + 3
// (G0 = first row / 32); the groups that share a block form a run, moved as
// one box and held in shared memory as [k][w][32] from position pos (in
// groups).  Run of the tile's group q: its position and width.
__device__ __forceinline__ void p_run(int G0, int q, int gp, int &pos, int &w)
{
    const int gg = (G0 + q) % gp;             // group within its block
    pos = q > gg ? q - gg : 0;
    const int gs = gg - (q - pos);            // the run's first group within the block
    w = min(4 - pos, gp - gs);
}

// The runs of one tile: a run starts at the tile's first group and at every
// group that opens a block; on[q] marks a run starting at group q that lies
// in the vector (blocks past the last are not moved).
struct PRuns {
    bool on[4];
    int w[4], gg[4], c2[4];
    uint32_t bytes;                           // bytes of one operand's boxes
};

__device__ __forceinline__ void p_runs(int G0, int gp, int nblk, PRuns &r)
{
    r.bytes = 0;
    #pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int Gq = G0 + q, c2 = Gq / gp, gg = Gq - c2 * gp;
        r.on[q] = (q == 0 || gg == 0) && c2 < nblk;
        r.w[q] = min(4 - q, gp - gg);
        r.gg[q] = gg;
        r.c2[q] = c2;
        if (r.on[q]) r.bytes += (uint32_t)r.w[q] * 2048u;
    }
}

template <bool F16>
__global__ void __launch_bounds__(kPThreads, 1)
tc32p_level_kernel(Tc32pArgs g, const __grid_constant__ Tc32pMaps mp)
{
    if (g.gate && *g.gate) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int NT = g.NT, KS = g.KS;
    const int bstep = 2 * NT * 32;                              // bytes of one K step of B (hi + lo)
    unsigned char *Bs = smem;
    unsigned char *slots = Bs + (size_t)KS * bstep;             // 1024-byte aligned (NT % 16 == 0)
    const int S = g.nslots;
    unsigned char *planes = slots + S * kPSlab;
    float *stage = reinterpret_cast<float *>(planes + kPPlanes * kPPlane);     // the epilogue region
    const size_t ebytes = (size_t)g.ering * g.echunk;
    float *binv_s = stage + (ebytes > kPStageBytes ? ebytes : kPStageBytes) / 4;
    uint64_t *full = reinterpret_cast<uint64_t *>(binv_s + 256);
    uint64_t *empty = full + kPSlotsMax;
    uint64_t *pfull = empty + kPSlotsMax;
    uint64_t *pfree = pfull + kPPlanes;
    uint64_t *accfull = pfree + kPPlanes;
    uint64_t *accempty = accfull + 2;
    uint64_t *efull = accempty + 2;
    uint64_t *eempty = efull + kPERingMax;
    uint64_t *sready = eempty + kPERingMax;                     // a chunk's four quarters written
    uint64_t *bready = sready + kPERingMax;
    uint64_t *drain = bready + 1;                               // products in flight at an abort
    volatile int *abort_flag = reinterpret_cast<volatile int *>(drain + 1);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(drain + 1) + 1;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;
    const int niter = (g.tiles - (int)blockIdx.x + G - 1) / G;  // tiles of this CTA
    const int nsteps = niter * KS;
    const bool kmajor = (g.a_sk == 1);
    const int Mi32 = (int)g.Mi;
    auto rowoff = [&](int m) -> i64 {
        const int mq = m / Mi32;
        return (i64)(m - mq * Mi32) * g.s1 + (i64)mq * g.s2;
    };
    auto vgated = [&](int z) -> bool { return g.vgate && g.vgate[(i64)z * g.vgate_stride]; };
    // points fastest: the runs of a tile (computed once per tile, so the
    // lanes that move boxes spend no divisions per box), their bytes, and
    // the boxes of one operand at k (or n) offset kk
    auto run_boxes = [&](unsigned char *dst, const PRuns &r, const CUtensorMap *maps, bool vec, int kk, int z,
                         uint64_t *bar) {
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (!r.on[q]) continue;
            if (vec) tma_load_5d(dst + q * 2048, &maps[r.w[q] - 1], 0, r.gg[q], kk, r.c2[q], z, bar);
            else tma_load_4d(dst + q * 2048, &maps[r.w[q] - 1], 0, r.gg[q], kk, r.c2[q], bar);
        }
    };
    auto fail = [&]() {
        *abort_flag = 1;
        if (g.err) atomicExch(g.err, 5);
    };

    if (tid == 0) {
        // the 64-byte swizzle of the boxes repeats every 512 bytes of shared memory
        if (smem_addr(slots) & 511) { if (g.err) atomicExch(g.err, 5); }
        for (int i = 0; i < S; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], kPConv); }
        for (int i = 0; i < kPPlanes; ++i) { mbar_init(&pfull[i], kPConv); mbar_init(&pfree[i], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&accfull[b], 1); mbar_init(&accempty[b], 32 * kPEpiWarps); }
        for (int i = 0; i < kPERingMax; ++i) {
            mbar_init(&efull[i], 1);
            mbar_init(&eempty[i], 1);
            mbar_init(&sready[i], 4);
        }
        mbar_init(bready, 1);
        mbar_init(drain, 1);
        *abort_flag = 0;
        mbar_init_fence();
        mbar_arrive_expect_tx(bready, (uint32_t)(KS * bstep));
        const unsigned char *src = reinterpret_cast<const unsigned char *>(g.bsplit);
        for (int ks = 0; ks < KS; ++ks) bulk_g2s(Bs + (size_t)ks * bstep, src + (size_t)ks * bstep, bstep, bready);
    }
    if (warp == kPMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tslot)), "r"(2 * kPAccCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int i = tid; i < 256; i += kPThreads) binv_s[i] = (F16 && g.binv && i < NT) ? g.binv[i] : 1.0f;
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *tslot;

    if (warp < kPConv / 32) {
        // ------------------------------------------------------ converters --
        const int row = tid & (kPM - 1), h = tid >> 7;
        const int poff = (row >> 3) * 256 + h * 128 + (row & 7) * 16;
        const int sw = (row >> 1) & 3;
        int ks = 0, it = 0;
        float xs = 1.0f;
        if (F16 && nsteps > 0) xs = p_pow2(p_scale_exp(g.xmax[(int)blockIdx.x / g.mtiles]));
        // points fastest: this row's place in the slab's runs
        int coff = 0, kstr = 0;
        auto crun = [&](int i) {
            if (kmajor) return;
            const int tau = (int)blockIdx.x + i * G, z = tau / g.mtiles;
            int pos, w;
            p_run(((tau - z * g.mtiles) * kPM) >> 5, row >> 5, g.gp, pos, w);
            coff = pos * 512 + ((row >> 5) - pos) * 32 + (row & 31);
            kstr = w * 32;
        };
        if (nsteps > 0) crun(0);
        int fs = 0, p = 0;                      // slot and plane of the next step
        uint32_t fph = 0, pphase = 0;
        // two K steps per pass: one fence and one round of arrivals for both
        for (int q = 0; q < nsteps; q += 2) {
            const int nu = (q + 1 < nsteps) ? 2 : 1;
            uint32_t hw[2][4], lw[2][4];
            int used[2];
            #pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (u >= nu) break;
                if (!*abort_flag && !mbar_wait(&full[fs], fph)) fail();
                const unsigned char *st = slots + fs * kPSlab;
                float x[8];
                if (kmajor) {
                    // the box's 64-byte swizzle: 16-byte piece c of row r at c ^ ((r >> 1) & 3)
                    const float4 a = *reinterpret_cast<const float4 *>(st + row * 64 + 16 * ((2 * h) ^ sw));
                    const float4 b = *reinterpret_cast<const float4 *>(st + row * 64 + 16 * ((2 * h + 1) ^ sw));
                    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
                    x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
                } else {
                    // runs [16 k][w][32 points]
                    const float *sf = reinterpret_cast<const float *>(st) + coff;
                    #pragma unroll
                    for (int j = 0; j < 8; ++j) x[j] = sf[(8 * h + j) * kstr];
                }
                #pragma unroll
                for (int j = 0; j < 4; ++j) p_cut2<F16>(x[2 * j], x[2 * j + 1], xs, hw[u][j], lw[u][j]);
                used[u] = fs;
                if (++fs == S) { fs = 0; fph ^= 1u; }
                if (++ks == KS) {
                    ks = 0;
                    ++it;
                    if (F16 && it < niter) xs = p_pow2(p_scale_exp(g.xmax[((int)blockIdx.x + it * G) / g.mtiles]));
                    if (it < niter) crun(it);
                }
            }
            #pragma unroll
            for (int u = 0; u < 2; ++u)
                if (u < nu) mbar_arrive(&empty[used[u]]);
            #pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (u >= nu) break;
                if (q + u >= kPPlanes && !*abort_flag && !mbar_wait(&pfree[p], pphase ^ 1u)) fail();
                unsigned char *pl = planes + p * kPPlane;
                *reinterpret_cast<uint4 *>(pl + poff) = make_uint4(hw[u][0], hw[u][1], hw[u][2], hw[u][3]);
                *reinterpret_cast<uint4 *>(pl + kPPlane / 2 + poff) = make_uint4(lw[u][0], lw[u][1], lw[u][2], lw[u][3]);
                if (++p == kPPlanes) { p = 0; pphase ^= 1u; }
            }
            fence_proxy_async_smem();
            int pa = p - nu;
            if (pa < 0) pa += kPPlanes;
            for (int u = 0; u < nu; ++u) {
                mbar_arrive(&pfull[pa]);
                if (++pa == kPPlanes) pa = 0;
            }
        }
    } else if (warp == kPLoadWarp) {
        // ------------------------------------------------------ load lane --
        if (lane == 0) {
            int pit = 0, pks = 0, pz = 0, pm0 = 0;
            bool pskip = false;
            PRuns pr;
            auto ptile = [&]() {
                const int tau = (int)blockIdx.x + pit * G;
                pz = tau / g.mtiles;
                pm0 = (tau - pz * g.mtiles) * kPM;
                pskip = vgated(pz);
                if (!kmajor) p_runs(pm0 >> 5, g.gp, g.nblk, pr);
            };
            if (nsteps > 0) ptile();
            int prod = 0, sl = 0;
            uint32_t rnd = 0;                 // parity of the ring round
            for (; prod < nsteps && !*abort_flag; ++prod) {
                // the load lanes' waits suspend until the phase completes (one
                // thread each: the spin of a lone lane costs the other warps of
                // its sub-partition issue slots; measured 0.16 -> 0.14 ms on a
                // points-fastest level).  Waits of warps whose lanes can diverge
                // inside the wait loop keep spinning: suspended diverged lanes
                // stalled the converters until their bounded waits expired.
                if (prod >= S && !mbar_wait_timed(&empty[sl], rnd ^ 1u)) {
                    fail();
                    break;
                }
                unsigned char *dst = slots + sl * kPSlab;
                if (pskip) {
                    mbar_arrive(&full[sl]);   // a stopped vector: nothing to load
                } else {
                    if (kmajor) {
                        mbar_arrive_expect_tx(&full[sl], (uint32_t)kPSlab);
                        tma_load_3d(dst, &mp.a[0], pks * 16, pm0, pz, &full[sl]);
                    } else {
                        mbar_arrive_expect_tx(&full[sl], pr.bytes);
                        run_boxes(dst, pr, mp.a, true, pks * 16, pz, &full[sl]);
                    }
                }
                if (++sl == S) { sl = 0; rnd ^= 1u; }
                if (++pks == KS) {
                    pks = 0;
                    if (++pit < niter) ptile();
                }
            }
            // the copies in flight land before the shared memory goes
            for (int q = prod - S < 0 ? 0 : prod - S; q < prod; ++q)
                mbar_wait_timed(&full[q % S], (uint32_t)((q / S) & 1), 200000000ull);
        }
        __syncwarp();
    } else if (warp == kPELoadWarp) {
        // ---------------------------------------- epilogue operands' lane --
        // points fastest: per tile and 16-column chunk, the accumulated output
        // (and for the diagonal term V and X) as the tile's runs
        if (lane == 0 && g.ering > 0) {
            const int nch = (g.N + 15) / 16;
            const bool dg = g.diagV != nullptr;
            const uint32_t piece = 4 * 2048;
            int cc = 0, sl = 0;
            uint32_t rnd = 0;
            PRuns er;
            for (int it = 0; it < niter && !*abort_flag; ++it) {
                const int tau = (int)blockIdx.x + it * G;
                const int z = tau / g.mtiles, m0 = (tau - z * g.mtiles) * kPM;
                const bool skip = vgated(z);
                p_runs(m0 >> 5, g.gp, g.nblk, er);
                const uint32_t tx = (g.accumulate ? er.bytes : 0u) + (dg ? 2 * er.bytes : 0u);
                for (int ch = 0; ch < nch; ++ch, ++cc) {
                    if (cc >= g.ering && !mbar_wait_timed(&eempty[sl], rnd ^ 1u)) {
                        fail();
                        break;
                    }
                    unsigned char *dst = reinterpret_cast<unsigned char *>(stage) + (size_t)sl * g.echunk;
                    if (skip || (!g.accumulate && !dg)) {
                        mbar_arrive(&efull[sl]);
                    } else {
                        mbar_arrive_expect_tx(&efull[sl], tx);
                        if (g.accumulate) run_boxes(dst, er, mp.c, true, ch * 16, z, &efull[sl]);
                        if (dg) {
                            run_boxes(dst + piece, er, mp.v, false, ch * 16, z, &efull[sl]);
                            run_boxes(dst + 2 * piece, er, mp.a, true, ch * 16, z, &efull[sl]);
                        }
                    }
                    if (++sl == g.ering) { sl = 0; rnd ^= 1u; }
                }
            }
            // the copies in flight land before the shared memory goes
            for (int q = cc - g.ering < 0 ? 0 : cc - g.ering; q < cc; ++q)
                mbar_wait_timed(&efull[q % g.ering], (uint32_t)((q / g.ering) & 1), 200000000ull);
        }
        __syncwarp();
    } else if (warp == kPMmaWarp) {
        // -------------------------------------------------------- MMA lane --
        if (lane == 0) {
            const uint32_t idesc = F16 ? idesc_f16(NT) : idesc_bf16(NT);
            if (!mbar_wait_timed(bready, 0)) fail();
            int q = 0, it = 0;
            for (; it < niter && !*abort_flag; ++it) {
                const int b = it & 1;
                if (it >= 2 && !mbar_wait(&accempty[b], (uint32_t)(((it >> 1) - 1) & 1))) { fail(); break; }
                for (int ks = 0; ks < KS; ++ks, ++q) {
                    const int pp = q % kPPlanes;
                    if (!mbar_wait(&pfull[pp], (uint32_t)((q / kPPlanes) & 1))) { fail(); break; }
                    fence_after();
                    const unsigned char *Ab = planes + pp * kPPlane;
                    const uint64_t a_hi = smem_desc(smem_addr(Ab), 128, 256);
                    const uint64_t a_lo = smem_desc(smem_addr(Ab + kPPlane / 2), 128, 256);
                    const unsigned char *Bk = Bs + (size_t)ks * bstep;
                    const uint64_t b_hi = smem_desc(smem_addr(Bk), 128, 256);
                    const uint64_t b_lo = smem_desc(smem_addr(Bk + NT * 32), 128, 256);
                    const uint32_t d = tbase + (uint32_t)(b * kPAccCols);
                    tc_mma(d, a_hi, b_hi, idesc, ks > 0 ? 1u : 0u);
                    tc_mma(d, a_hi, b_lo, idesc, 1u);
                    tc_mma(d, a_lo, b_hi, idesc, 1u);
                    tc_commit(&pfree[pp]);
                }
                if (*abort_flag) break;
                tc_commit(&accfull[b]);
            }
            // every product has completed before the TMEM and the planes go
            tc_commit(drain);
            mbar_wait_timed(drain, 0, 200000000ull);
        }
        __syncwarp();
    } else {
        // -------------------------------------------------------- epilogue --
        const int qd = warp & 3;                 // TMEM lanes 32 qd .. 32 qd + 31 (warp % 4)
        const int ew = warp - kPConv / 32;       // 0 .. kPEpiWarps - 1
        const int hc = ew >> 2;                  // this warp's half of the columns
        float *stg0 = stage + ew * 2 * kPStage;
        const int nch = (g.N + 15) / 16;
        const uint32_t lane_base = (uint32_t)(qd * 32) << 16;
        int nstore = 0;                          // TMA stores issued by this warp
        for (int it = 0; it < niter; ++it) {
            const int b = it & 1;
            const int tau = (int)blockIdx.x + it * G;
            const int z = tau / g.mtiles, m0 = (tau - z * g.mtiles) * kPM;
            bool ok = !*abort_flag;
            if (ok && !mbar_wait_sleep(&accfull[b], (uint32_t)((it >> 1) & 1), 256)) {
                fail();
                ok = false;
            }
            ok = __all_sync(0xffffffffu, ok);
            fence_after();
            if (ok && !vgated(z)) {
                const float xinv = F16 ? p_pow2(-p_scale_exp(g.xmax[z])) : 1.0f;
                const float shift = g.shiftv ? g.shiftv[z] : g.shift;
                const float *Vd = g.diagV;
                const float *Xd = g.diagX + (i64)z * g.dx_sz;
                float *C = g.C + (i64)z * g.c_sz;
                const int r = qd * 32 + lane;
                const int m = m0 + r;
                const float rs = (g.rowscale && m < g.M) ? g.rowscale[m % Mi32] : 1.0f;
                const float sc = g.alpha * rs * xinv;
                if (g.tstore) {
                    // rows contiguous along n, nothing to add: each 32 x 16 block
                    // is scaled into one of the warp's two stages (64-byte
                    // swizzle) and stored by one TMA copy; rows past the vector's
                    // last are clipped by the copy
                    const int sw = (lane >> 1) & 3;
                    const bool rows_in = m0 + qd * 32 < g.M;
                    for (int ch = hc; ch < nch; ch += 2) {
                        float v[16];
                        tmem_ld16(tbase + lane_base + (uint32_t)(b * kPAccCols + ch * 16), v);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        float *stg = stg0 + (nstore & 1) * kPStage;
                        if (nstore >= 2) {
                            if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                            __syncwarp();
                        }
                        #pragma unroll
                        for (int j4 = 0; j4 < 4; ++j4) {
                            const float *cs = binv_s + ch * 16 + 4 * j4;
                            *reinterpret_cast<float4 *>(stg + lane * 16 + 4 * (j4 ^ sw)) =
                                make_float4(sc * cs[0] * v[4 * j4], sc * cs[1] * v[4 * j4 + 1],
                                            sc * cs[2] * v[4 * j4 + 2], sc * cs[3] * v[4 * j4 + 3]);
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0 && rows_in) {
                            tma_store_3d(&mp.c[0], stg, ch * 16, m0 + qd * 32, z);
                            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                        }
                        ++nstore;
                    }
                } else if (g.c_sn == 1) {
                    // rows contiguous along n with a diagonal term or an output
                    // to add: 32 x 16 blocks through the warp's stage, finished
                    // as 64-byte row pieces
                    const int f = lane & 3;
                    const int sw = (lane >> 1) & 3;
                    float *stg = stg0;
                    for (int ch = hc; ch < nch; ch += 2) {
                        float v[16];
                        tmem_ld16(tbase + lane_base + (uint32_t)(b * kPAccCols + ch * 16), v);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        #pragma unroll
                        for (int j4 = 0; j4 < 4; ++j4)
                            *reinterpret_cast<float4 *>(stg + lane * 16 + 4 * (j4 ^ sw)) =
                                make_float4(sc * v[4 * j4], sc * v[4 * j4 + 1], sc * v[4 * j4 + 2], sc * v[4 * j4 + 3]);
                        __syncwarp();
                        const int n = ch * 16 + 4 * f;
                        const float4 cs = *reinterpret_cast<const float4 *>(binv_s + n);
                        #pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int rr = 8 * u + (lane >> 2);
                            const float4 o = *reinterpret_cast<const float4 *>(stg + rr * 16 + 4 * (f ^ ((rr >> 1) & 3)));
                            const int mm = m0 + qd * 32 + rr;
                            if (mm >= g.M || n >= g.N) continue;
                            const i64 pp = rowoff(mm) + n;
                            float4 out = make_float4(o.x * cs.x, o.y * cs.y, o.z * cs.z, o.w * cs.w);
                            if (Vd) {
                                const float4 dv = __ldg(reinterpret_cast<const float4 *>(Vd + pp));
                                const float4 dx = __ldg(reinterpret_cast<const float4 *>(Xd + pp));
                                out.x = fmaf(g.alpha * (dv.x - shift), dx.x, out.x);
                                out.y = fmaf(g.alpha * (dv.y - shift), dx.y, out.y);
                                out.z = fmaf(g.alpha * (dv.z - shift), dx.z, out.z);
                                out.w = fmaf(g.alpha * (dv.w - shift), dx.w, out.w);
                            }
                            if (g.accumulate) {
                                const float4 cy = *reinterpret_cast<const float4 *>(C + pp);
                                out.x += cy.x; out.y += cy.y; out.z += cy.z; out.w += cy.w;
                            }
                            *reinterpret_cast<float4 *>(C + pp) = out;
                        }
                        __syncwarp();
                    }
                } else {
                    // points fastest: per 16-column chunk of this warp's half, the
                    // operands wait in the ring as the tile's runs [16 n][w][32
                    // points]; the result overwrites the output's place and, once
                    // the four quarters are written, the first quarter's lane 0
                    // stores the runs (blocks past the last are not stored) and
                    // releases the slot when the copies have read it
                    const float *cs = binv_s;
                    const int G0 = m0 >> 5;
                    int pos, w;
                    p_run(G0, qd, g.gp, pos, w);
                    const int ebase = pos * 512 + (qd - pos) * 32 + lane, nstr = w * 32;
                    PRuns er;
                    if (qd == 0) p_runs(G0, g.gp, g.nblk, er);
                    const int cc0 = it * nch, q0 = cc0 / g.ering, r0 = cc0 - q0 * g.ering;
                    for (int ch = hc; ch < nch; ch += 2) {
                        // ring slot and round of chunk it * nch + ch
                        int sl = r0 + ch, rq = q0;
                        while (sl >= g.ering) { sl -= g.ering; ++rq; }
                        const uint32_t par = (uint32_t)(rq & 1);
                        float v[16];
                        tmem_ld16(tbase + lane_base + (uint32_t)(b * kPAccCols + ch * 16), v);
                        bool eok = !*abort_flag && mbar_wait(&efull[sl], par);
                        eok = __all_sync(0xffffffffu, eok);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        if (!eok) { fail(); break; }
                        float *cbuf = stage + (size_t)sl * (g.echunk / 4);
                        float *cb = cbuf + ebase;
                        #pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int n = ch * 16 + j;
                            const int idx = j * nstr;
                            float out = v[j] * (sc * cs[n < 256 ? n : 0]);
                            if (g.accumulate) out += cb[idx];
                            if (Vd) out = fmaf(g.alpha * (cb[2048 + idx] - shift), cb[4096 + idx], out);
                            cb[idx] = out;
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            mbar_arrive(&sready[sl]);
                            if (qd == 0) {
                                if (!mbar_wait(&sready[sl], par)) {
                                    fail();
                                } else {
                                    #pragma unroll
                                    for (int q = 0; q < 4; ++q) {
                                        if (!er.on[q]) continue;
                                        tma_store_5d(&mp.c[er.w[q] - 1], cbuf + q * 512, 0, er.gg[q], ch * 16,
                                                     er.c2[q], z);
                                        ++nstore;
                                    }
                                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                                    mbar_arrive(&eempty[sl]);
                                }
                            }
                        }
                        __syncwarp();
                        if (*abort_flag) break;
                    }
                }
            } else if (ok && g.ering > 0) {
                // a stopped vector: its ring chunks are released unread (the
                // quarters still mark each chunk so the phases stay in step)
                const int cc0 = it * nch, q0 = cc0 / g.ering, r0 = cc0 - q0 * g.ering;
                for (int ch = hc; ch < nch; ch += 2) {
                    int sl = r0 + ch, rq = q0;
                    while (sl >= g.ering) { sl -= g.ering; ++rq; }
                    const uint32_t par = (uint32_t)(rq & 1);
                    if (lane == 0) {
                        mbar_arrive(&sready[sl]);
                        if (qd == 0) {
                            if (mbar_wait(&sready[sl], par) && mbar_wait(&efull[sl], par)) mbar_arrive(&eempty[sl]);
                            else fail();
                        }
                    }
                    __syncwarp();
                }
            }
            fence_before();
            mbar_arrive(&accempty[b]);
        }
        // the stage buffers are read and the stores complete before the CTA ends
        if (lane == 0 && nstore > 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }

    // B copies have landed before the shared memory goes (an abort may skip
    // the load lane's wait on them)
    if (tid == 0) mbar_wait_timed(bready, 0, 200000000ull);
    fence_before();
    __syncthreads();
    if (warp == kPMmaWarp)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(2 * kPAccCols) : "memory");
}

// Per-vector max |x| as float bits (atomicMax on the non-negative bit
// patterns); out[] must be zero before the launch.  Stopped vectors are
// skipped.
__global__ void absmax_bits_kernel(const float *__restrict__ X, i64 n, i64 vstride, unsigned *out,
                                   const int *gate, const int *vgate, int vgstride)
{
    if (gate && *gate) return;
    const int z = blockIdx.y;
    if (vgate && vgate[(i64)z * vgstride]) return;
    const float *x = X + (i64)z * vstride;
    float mx = 0.0f;
    const i64 n4 = n / 4;
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n4; i += (i64)gridDim.x * blockDim.x) {
        const float4 v = __ldg(x4 + i);
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
    for (i64 i = 4 * n4 + blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        mx = fmaxf(mx, fabsf(x[i]));
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (threadIdx.x == 0) atomicMax(out + z, __float_as_uint(mx));
    }
}

// FP16 hi/lo planes of B(k, n) = H(n, k) (H nout x nout, column-major) with
// every column n scaled by 2^e_n (max_k |H(n, k)| 2^e_n in [2^14, 2^15)),
// canonical layout [KS][hi, lo][NT x 16], and binv[n] = 2^-e_n.  One block
// per column of the tile (columns past nout stay zero, binv 1).
__global__ void split_b16_kernel(int nout, int NT, const float *__restrict__ H, uint16_t *__restrict__ out,
                                 float *__restrict__ binv)
{
    const int n = blockIdx.x;
    if (n >= nout) { if (threadIdx.x == 0) binv[n] = 1.0f; return; }
    float mx = 0.0f;
    for (int k = threadIdx.x; k < nout; k += blockDim.x) mx = fmaxf(mx, fabsf(H[n + (i64)k * nout]));
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ float red[32];
    __shared__ float s_scale;
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
        const int e = p_scale_exp(__float_as_uint(m));
        s_scale = p_pow2(e);
        binv[n] = p_pow2(-e);
    }
    __syncthreads();
    const float s = s_scale;
    for (int k = threadIdx.x; k < nout; k += blockDim.x) {
        const float v = H[n + (i64)k * nout] * s;
        const __half hh = __float2half_rn(v);
        const __half ll = __float2half_rn(v - __half2float(hh));
        const int ks = k / 16, kk = k % 16;
        const size_t base = (size_t)ks * 2 * NT * 16;
        const size_t off = (size_t)(n >> 3) * 128 + (size_t)(kk >> 3) * 64 + (size_t)(n & 7) * 8 + (kk & 7);
        out[base + off] = __half_as_ushort(hh);
        out[base + (size_t)NT * 16 + off] = __half_as_ushort(ll);
    }
}

// ------------------------------------------------------------------ host --

// Epilogue operand ring of a points-fastest level: slots of 8 KB per operand
// (the output, and V and X for the diagonal term), as many as fit (at most
// kPERingMax, at least two).
static int p_ring(int NT, int KS, bool diag, int *echunk)
{
    const size_t fixed = p_fixed_bytes(NT, KS, kPSlotsM);
    const int chunk = 8192 * (diag ? 3 : 1);
    if (echunk) *echunk = chunk;
    if (fixed >= (size_t)kPMaxSmem) return 0;
    const size_t room = (size_t)kPMaxSmem - fixed;
    int r = (int)(room / chunk);
    return r > kPERingMax ? kPERingMax : r;
}

static bool p_fits(int NT, int KS, bool kmajor, bool diag)
{
    if (kmajor) return p_smem_bytes(NT, KS, kPSlotsMax, 0) <= (size_t)kPMaxSmem;
    return p_ring(NT, KS, diag, nullptr) >= 2;
}

void tc16_free(scalit_ctx *c)
{
    for (int l = 0; l < SCALIT_FMAX; ++l) {
        if (c->tc16[l].dig) cudaFree(c->tc16[l].dig);
        if (c->tc16[l].cscale) cudaFree(c->tc16[l].cscale);
        c->tc16[l] = TcLevelData{};
    }
    if (c->xmax) { cudaFree(c->xmax); c->xmax = nullptr; }
}

// FP16 planes and column scales of every level matrix that one persistent
// tile holds (after load).
int tc16_prepare(scalit_ctx *c)
{
    const Layout &L = c->L;
    tc16_free(c);
    SC_CUDA(cudaMalloc(&c->xmax, sizeof(unsigned) * kPMaxVec));
    for (int l = 0; l < L.nlev; ++l) {
        if (L.ndvr && l == L.nlev - 1) continue;
        const int nout = L.n[l];
        const int NT = (nout + 15) / 16 * 16, KS = (nout + 15) / 16;
        if (NT > 256 || !p_fits(NT, KS, L.dim[l] == 1, false)) continue;
        TcLevelData &t = c->tc16[l];
        const size_t nel = (size_t)KS * 2 * NT * 16;
        SC_CUDA(cudaMalloc(&t.dig, nel * sizeof(uint16_t)));
        SC_CUDA(cudaMalloc(&t.cscale, sizeof(float) * NT));
        SC_CUDA(cudaMemsetAsync(t.dig, 0, nel * sizeof(uint16_t), c->stream));
        split_b16_kernel<<<NT, 128, 0, c->stream>>>(nout, NT, c->H0f + L.h0s[l], t.dig, t.cscale);
        SC_CHECK_LAUNCH();
        t.NT = NT; t.ntiles = 1; t.KS = KS; t.usable = 1;
    }
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

// The persistent kernel applies to level l when one tile holds the level
// matrix (single N tile, shared memory) and the operand's rows allow 16-byte
// copies.  f16 selects the FP16 planes, else the BF16 planes of tc_fp32.cu.
bool tc32p_usable(const scalit_ctx *c, int l, bool f16, bool diag)
{
    const Layout &L = c->L;
    if (L.ndvr && l == L.nlev - 1) return false;
    const TcLevelData &t = f16 ? c->tc16[l] : c->tc32[l];
    if (!t.usable || t.ntiles != 1 || !p_fits(t.NT, t.KS, L.dim[l] == 1, diag)) return false;
    if (f16 && !c->xmax) return false;
    const int nout = L.n[l];
    const i64 nin = L.dim[l], N = L.N;
    if (N % 4 || nout % 4) return false;
    // grid points fastest within blocks of nin: 32-point groups stay in a block
    if (nin > 1 && nin % 32) return false;
    return true;
}

// cuTensorMapEncodeTiled from the driver (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Tensor map (FP32 or FP64 elements) of rank r over base with the given
// extents (elements), strides of dimensions 1.. (bytes) and box; zero fill
// outside.
int tma_encode(CUtensorMap *map, const void *base, bool f64, int rank, const cuuint64_t *dims,
               const cuuint64_t *strides, const cuuint32_t *box, CUtensorMapSwizzle swz)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return SCALIT_ECUDA; }
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = fn(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                          (cuuint32_t)rank, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return SCALIT_ECUDA; }
    return 0;
}

static int encode_map(CUtensorMap *map, const float *base, int rank, const cuuint64_t *dims,
                      const cuuint64_t *strides, const cuuint32_t *box, CUtensorMapSwizzle swz)
{
    return tma_encode(map, base, false, rank, dims, strides, box, swz);
}

// Per-vector scales of X (FP16 form): zero the slots, then one max pass.
int tc16_scales(const scalit_ctx *c, const float *X, int nvec, const int *gate, cudaStream_t s,
                const int *vgate, int vstride)
{
    if (nvec > kPMaxVec) { set_error("more than %d vectors in one FP16 tensor-core launch", kPMaxVec); return SCALIT_EINVAL; }
    SC_CUDA(cudaMemsetAsync(c->xmax, 0, sizeof(unsigned) * nvec, s));
    if ((reinterpret_cast<uintptr_t>(X) & 15) || (c->L.N % 4)) { set_error("FP16 tensor-core operand not 16-byte aligned"); return SCALIT_EINVAL; }
    const i64 n4 = c->L.N / 4;
    int bx = (int)((n4 + 255) / 256);
    const int cap = 152 * 8 / (nvec < 8 ? nvec : 8) + 1;
    if (bx > cap) bx = cap;
    absmax_bits_kernel<<<dim3(bx, nvec), 256, 0, s>>>(X, c->L.N, c->L.N, c->xmax, gate, vgate, vstride);
    SC_CHECK_LAUNCH();
    return 0;
}

int tc32p_level_apply(const scalit_ctx *c, int l, bool f16, const float *X, float *Y, int accumulate,
                      const float *diagV, float shift, float alpha, const int *gate, cudaStream_t s, int nvec,
                      const float *shiftv, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const TcLevelData &t = f16 ? c->tc16[l] : c->tc32[l];
    if (!tc32p_usable(c, l, f16, diagV != nullptr)) {
        set_error("level %d has no persistent tensor-core plan", l + 1);
        return SCALIT_EUNSUP;
    }
    if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Y) & 15)) {
        set_error("persistent tensor-core operands not 16-byte aligned");
        return SCALIT_EINVAL;
    }
    if (nvec > kPMaxVec) { set_error("more than %d vectors in one persistent launch", kPMaxVec); return SCALIT_EINVAL; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    Tc32pArgs g{};
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
    g.mtiles = (g.M + kPM - 1) / kPM;
    const i64 tiles = (i64)g.mtiles * nvec;
    if (tiles > 2147483647LL) { set_error("level %d: too many tiles", l + 1); return SCALIT_EINVAL; }
    g.tiles = (int)tiles;
    g.C = Y; g.c_sz = N;
    g.accumulate = accumulate; g.alpha = alpha;
    g.diagV = diagV; g.diagX = X; g.dx_sz = N; g.shift = shift; g.shiftv = shiftv;
    g.vgate = vgate; g.vgate_stride = vstride;
    g.gate = gate; g.err = c->tc_err;
    g.bsplit = reinterpret_cast<const uint4 *>(t.dig);
    g.binv = f16 ? t.cscale : nullptr;
    g.xmax = f16 ? c->xmax : nullptr;
    g.tstore = (g.c_sn == 1 && !accumulate && !diagV) ? 1 : 0;

    // the grid operand: [vector][row][k] boxes of 16 k x 128 rows (64-byte
    // swizzle), the level-1 output for TMA stores: [vector][row][n] boxes of
    // 16 n x 32 rows; points fastest: the grid operand, the output (loaded to
    // accumulate, stored back) and V (no vector dimension) as
    // [vector][block][k][group][point] boxes of 32 points x w groups x 16 k
    Tc32pMaps mp;
    memset(&mp, 0, sizeof(mp));
    int rc = 0;
    if (nin == 1) {
        const cuuint64_t dims[3] = {(cuuint64_t)nout, (cuuint64_t)blk, (cuuint64_t)nvec};
        const cuuint64_t str[2] = {(cuuint64_t)nout * 4, (cuuint64_t)N * 4};
        const cuuint32_t box[3] = {16, kPM, 1};
        rc = encode_map(&mp.a[0], X, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_64B);
        if (!rc && g.tstore) {
            const cuuint32_t boxc[3] = {16, 32, 1};
            rc = encode_map(&mp.c[0], Y, 3, dims, str, boxc, CU_TENSOR_MAP_SWIZZLE_64B);
        }
    } else {
        const i64 gp = nin / 32;
        g.gp = (int)gp; g.nblk = (int)blk;
        const cuuint64_t dims[5] = {32, (cuuint64_t)gp, (cuuint64_t)nout, (cuuint64_t)blk, (cuuint64_t)nvec};
        const cuuint64_t str[4] = {128, (cuuint64_t)nin * 4, (cuuint64_t)nin * nout * 4, (cuuint64_t)N * 4};
        // every run is 4 groups wide when the blocks hold whole tiles
        const int wmin = (gp % 4 == 0) ? 4 : 1, wmax = gp < 4 ? (int)gp : 4;
        for (int w = wmin; w <= wmax && !rc; ++w) {
            const cuuint32_t box[5] = {32, (cuuint32_t)w, 16, 1, 1};
            rc = encode_map(&mp.a[w - 1], X, 5, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE);
            if (!rc) rc = encode_map(&mp.c[w - 1], Y, 5, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE);
            if (!rc && diagV) rc = encode_map(&mp.v[w - 1], diagV, 4, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE);
        }
        g.ering = p_ring(g.NT, g.KS, diagV != nullptr, &g.echunk);
    }
    if (rc) return rc;

    static int sms = 0, configured = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        SC_CUDA(cudaFuncSetAttribute(tc32p_level_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPMaxSmem));
        SC_CUDA(cudaFuncSetAttribute(tc32p_level_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPMaxSmem));
        configured = dev;
    }
    const int grid = (int)(tiles < sms ? tiles : sms);
    g.nslots = nin == 1 ? kPSlotsMax : kPSlotsM;
    const size_t smem = p_smem_bytes(g.NT, g.KS, g.nslots, (size_t)g.ering * g.echunk);
    if (f16) tc32p_level_kernel<true><<<grid, kPThreads, smem, s>>>(g, mp);
    else tc32p_level_kernel<false><<<grid, kPThreads, smem, s>>>(g, mp);
    SC_CHECK_LAUNCH();
    return 0;
}

}  // namespace sc
