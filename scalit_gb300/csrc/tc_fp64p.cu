// Persistent FP64 level products of H*X on the tcgen05 digit engine.
//
// The arithmetic is the digit scheme of tc_fp64.cu: with e_m the binary
// exponent of the largest |x| of grid row m and e_n that of column n of B,
//   A(m, k) = 2^e_m sum_{s=0..6} a_s 2^-7(s+1),  B(k, n) = 2^e_n sum_t b_t 2^-7(t+1),
// |a_s|, |b_t| <= 127 integers (exact in BF16), and the 28 digit pairs with
// s + t <= 6 accumulate into 7 FP32 group accumulators in TMEM (exact for
// groups 0..5 with K <= 160), recombined in 64-bit integers in the epilogue.
// The row exponents come from one pass over each level's rows before the
// level (rowexp_kernel), so every K slab can be cut as it arrives; the digits
// are those of tc_fp64.cu.
//
// The pipeline is that of tc_fp32p.cu: one CTA per SM walks tiles of 128
// grid rows x one N tile of at most 64 columns (7 x 64 TMEM columns), N tile
// fastest so that neighbouring CTAs share the grid operand's tile in L2.
//   load lane (warp 17)     per K step, a TMA tensor copy of the FP64 slab
//                           (16 k x 128 rows, 128-byte swizzle, or four 32-point
//                           x 16 k boxes when points are fastest) and a bulk copy
//                           of the step's 7 B digit planes, into one of
//                           kQSlots step slots ("full" / "empty" mbarriers; a slot
//                           is empty once the converters read its slab and the
//                           step's products read its B planes);
//   converters (warps 0-7)  cut the slab into 7 BF16 digit planes (K-major
//                           canonical layout) in one of kQPlanes plane slots;
//   MMA lane (warp 16)      issues the step's 28 products;
//   epilogue (warps 8-15)   recombine the groups, scale, add the diagonal term
//                           and the accumulated output, store; level-1 outputs
//                           leave by TMA from swizzled 32 x 8 stages.
// The accumulator is single (448 of 512 columns), so a tile's products start
// once the previous tile's epilogue has read it; loads and cuts run ahead.
// Every wait is bounded as in tc_fp32p.cu.
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda_bf16.h>

namespace sc {

static constexpr int kQM = 128;
static constexpr int kQConv = 256;
static constexpr int kQEpiWarps = 8;
static constexpr int kQThreads = kQConv + 32 * kQEpiWarps + 96;
static constexpr int kQMmaWarp = kQConv / 32 + kQEpiWarps;
static constexpr int kQLoadWarp = kQMmaWarp + 1;
static constexpr int kQELoadWarp = kQMmaWarp + 2;              // the epilogue operands' load lane
static constexpr int kQERingMax = 8;
static constexpr int kQDig = 7;
static constexpr int kQNTMax = 64;
static constexpr int kQSlabA = kQM * 16 * 8;                   // FP64 slab: 16 KB
static constexpr int kQBStepMax = kQDig * kQNTMax * 32;        // B digits of a K step: <= 14 KB
static constexpr int kQSlot = kQSlabA + kQBStepMax;            // 30 KB (a multiple of 1 KB)
static constexpr int kQSlots = 3;
static constexpr int kQPlane = kQDig * kQM * 32;               // A digit planes of a K step: 28 KB
static constexpr int kQPlanes = 3;
static constexpr int kQStage = 32 * 8;                         // doubles per epilogue stage (2 per warp)

struct Tc64pArgs {
    int M, K, KS, N, NT, ntn;   // rows per vector, contraction, K steps, output columns, N tile, N tiles
    int mtiles, tiles;          // M tiles per vector; tiles = mtiles x ntn x vectors
    i64 Mi, s1, s2, a_sk, c_sn;
    double *C; i64 c_sz;
    const double *rowscale;
    int accumulate;
    double alpha;
    const double *diagV;
    const double *diagX; i64 dx_sz;
    double shift;
    const double *shiftv;
    const int *vgate; int vgate_stride;
    const int *gate;
    int *err;
    const uint16_t *bdig;       // [ntile][ks][digit][NT x 16] canonical K-major
    const int *bexp;            // [ntile * NT] column exponents
    const int *rexp;            // per row of every vector (z M + m): binary exponent of the row's max |x|
    int tstore;                 // outputs contiguous along n, nothing to add: TMA stores
    int ering, echunk;          // points fastest: epilogue operand ring slots and bytes per slot
};

// Shared memory: step slots, plane slots, the epilogue region (level 1: two
// 32 x 8 stages per epilogue warp; otherwise the operand ring), barriers.
static constexpr size_t kQStageBytes = (size_t)kQEpiWarps * 2 * kQStage * 8;
static constexpr size_t kQFixed = (size_t)kQSlots * kQSlot + (size_t)kQPlanes * kQPlane +
                                  (2 * kQSlots + 2 * kQPlanes + 2 * kQERingMax + 4) * 8 + 16;
static constexpr int kQMaxSmem = 227 * 1024;

static size_t q_smem_bytes(size_t ebytes)
{
    return kQFixed + (ebytes > kQStageBytes ? ebytes : kQStageBytes);
}

// Epilogue operand ring of a points-fastest level: 8 KB per operand and
// 8-column chunk (the output, and V and X for the diagonal term).
static int q_ring(bool diag, int *echunk)
{
    const int chunk = 8192 * (diag ? 3 : 1);
    if (echunk) *echunk = chunk;
    int r = (int)(((size_t)kQMaxSmem - kQFixed) / chunk);
    return r > kQERingMax ? kQERingMax : r;
}

// Binary exponent e with |x| < 2^e (frexp's) from the bits of |x|; 0 for zero.
__device__ __forceinline__ int q_exp(unsigned long long bits)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex) return ex - 1022;
    const unsigned long long m = bits & 0x000FFFFFFFFFFFFFULL;
    return m ? (64 - __clzll(m)) - 1074 : 0;
}

// 49-bit fixed-point magnitude of |x| 2^(49 - e) (truncated), e >= exponent of x.
__device__ __forceinline__ unsigned long long q_fixed49(unsigned long long bits, int e)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long m = (bits & 0x000FFFFFFFFFFFFFULL) | (ex ? (1ULL << 52) : 0ULL);
    const int sh = (ex ? ex : 1) - 1075 + 49 - e;   // <= -4
    return (sh <= -64) ? 0ULL : (m >> (-sh));
}


__global__ void __launch_bounds__(kQThreads, 1)
tc64p_level_kernel(Tc64pArgs g, const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmC,
                   const __grid_constant__ CUtensorMap tmV, const __grid_constant__ CUtensorMap tmX)
{
    if (g.gate && *g.gate) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int NT = g.NT, KS = g.KS;
    const int bstep = kQDig * NT * 32;
    unsigned char *slots = smem;                                     // 1024-byte aligned
    unsigned char *planes = slots + kQSlots * kQSlot;
    double *stage = reinterpret_cast<double *>(planes + kQPlanes * kQPlane);
    const size_t ebytes = (size_t)g.ering * g.echunk;
    uint64_t *full = reinterpret_cast<uint64_t *>(reinterpret_cast<unsigned char *>(stage) +
                                                  (ebytes > kQStageBytes ? ebytes : kQStageBytes));
    uint64_t *empty = full + kQSlots;
    uint64_t *pfull = empty + kQSlots;
    uint64_t *pfree = pfull + kQPlanes;
    uint64_t *accfull = pfree + kQPlanes;
    uint64_t *accempty = accfull + 1;
    uint64_t *efull = accempty + 1;
    uint64_t *eempty = efull + kQERingMax;
    uint64_t *drain = eempty + kQERingMax;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(drain + 1);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(drain + 1) + 1;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;
    const int niter = (g.tiles - (int)blockIdx.x + G - 1) / G;
    const int nsteps = niter * KS;
    const bool kmajor = (g.a_sk == 1);
    const int Mi32 = (int)g.Mi;
    const int per_vec = g.mtiles * g.ntn;
    auto rowoff = [&](int m) -> i64 {
        const int mq = m / Mi32;
        return (i64)(m - mq * Mi32) * g.s1 + (i64)mq * g.s2;
    };
    auto vgated = [&](int z) -> bool { return g.vgate && g.vgate[(i64)z * g.vgate_stride]; };
    auto fail = [&]() {
        *abort_flag = 1;
        if (g.err) atomicExch(g.err, 6);
    };
    // tile -> vector, first row, N tile
    auto tile_of = [&](int it, int &z, int &m0, int &nt) {
        const int tau = (int)blockIdx.x + it * G;
        z = tau / per_vec;
        const int r = tau - z * per_vec;
        const int mt = r / g.ntn;
        nt = r - mt * g.ntn;
        m0 = mt * kQM;
    };

    if (tid == 0) {
        if (smem_addr(slots) & 1023) { if (g.err) atomicExch(g.err, 6); }
        for (int i = 0; i < kQSlots; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], kQConv + 1); }
        for (int i = 0; i < kQPlanes; ++i) { mbar_init(&pfull[i], kQConv); mbar_init(&pfree[i], 1); }
        mbar_init(accfull, 1);
        mbar_init(accempty, 32 * kQEpiWarps);
        for (int i = 0; i < kQERingMax; ++i) { mbar_init(&efull[i], 1); mbar_init(&eempty[i], 4); }
        mbar_init(drain, 1);
        *abort_flag = 0;
        mbar_init_fence();
    }
    if (warp == kQMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tslot)), "r"(512) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *tslot;

    if (warp < kQConv / 32) {
        // ------------------------------------------------------ converters --
        const int row = tid & (kQM - 1), h = tid >> 7;
        const int poff = (row >> 3) * 256 + h * 128 + (row & 7) * 16;
        int ks = 0, it = 0, fs = 0, p = 0;
        uint32_t fph = 0, pph = 0;
        // this thread's grid row's exponent (the digits are the row's 49-bit
        // fixed-point magnitudes, as in tc_fp64.cu)
        auto row_exp = [&](int it) -> int {
            int z, m0, nt;
            tile_of(it, z, m0, nt);
            return (m0 + row < g.M) ? g.rexp[(i64)z * g.M + m0 + row] : 0;
        };
        int e = nsteps > 0 ? row_exp(0) : 0;
        for (int q = 0; q < nsteps; ++q) {
            if (!*abort_flag && !mbar_wait(&full[fs], fph)) fail();
            const unsigned char *st = slots + fs * kQSlot;
            unsigned long long xb[8];
            if (kmajor) {
                // the box's 128-byte swizzle: 16-byte piece c of row r at c ^ (r & 7)
                #pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(st + row * 128 + 16 * ((4 * h + i) ^ (row & 7)));
                    xb[2 * i] = v.x;
                    xb[2 * i + 1] = v.y;
                }
            } else {
                const unsigned long long *sd = reinterpret_cast<const unsigned long long *>(st) + (row >> 5) * 512 + (row & 31);
                #pragma unroll
                for (int j = 0; j < 8; ++j) xb[j] = sd[(8 * h + j) * 32];
            }
            mbar_arrive(&empty[fs]);
            // the 49-bit magnitudes as 28 + 21 bits; digit s = bits 42-7s .. 48-7s
            uint32_t Fh[8], Fl[8], sg[8];
            #pragma unroll
            for (int j = 0; j < 8; ++j) {
                const unsigned long long F = q_fixed49(xb[j], e);
                Fh[j] = (uint32_t)(F >> 21);
                Fl[j] = (uint32_t)F & 0x1FFFFFu;
                sg[j] = (uint32_t)(xb[j] >> 32) & 0x80000000u;
            }
            if (q >= kQPlanes && !*abort_flag && !mbar_wait(&pfree[p], pph ^ 1u)) fail();
            unsigned char *pl = planes + p * kQPlane;
            #pragma unroll
            for (int s = 0; s < kQDig; ++s) {
                uint32_t w[4];
                #pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    const uint32_t d0 = s < 4 ? (Fh[j] >> (21 - 7 * s)) & 127u : (Fl[j] >> (42 - 7 * s)) & 127u;
                    const uint32_t d1 = s < 4 ? (Fh[j + 1] >> (21 - 7 * s)) & 127u : (Fl[j + 1] >> (42 - 7 * s)) & 127u;
                    // the digit as an exact float (2^23 + d - 2^23) with x's sign; its
                    // upper 16 bits are the BF16 digit
                    const uint32_t f0 = __float_as_uint(__uint_as_float(0x4B000000u | d0) - 8388608.0f) | sg[j];
                    const uint32_t f1 = __float_as_uint(__uint_as_float(0x4B000000u | d1) - 8388608.0f) | sg[j + 1];
                    w[j >> 1] = __byte_perm(f0, f1, 0x7632);
                }
                *reinterpret_cast<uint4 *>(pl + s * (kQM * 32) + poff) = make_uint4(w[0], w[1], w[2], w[3]);
            }
            fence_proxy_async_smem();
            mbar_arrive(&pfull[p]);
            if (++fs == kQSlots) { fs = 0; fph ^= 1u; }
            if (++p == kQPlanes) { p = 0; pph ^= 1u; }
            if (++ks == KS) {
                ks = 0;
                if (++it < niter) e = row_exp(it);
            }
        }
    } else if (warp == kQELoadWarp) {
        // ---------------------------------------- epilogue operands' lane --
        // points fastest: per tile and 8-column chunk, the accumulated output
        // (and for the diagonal term V and X) as four 32-point boxes each
        if (lane == 0 && g.ering > 0) {
            const int nck = NT / 8;
            const bool dg = g.diagV != nullptr;
            const uint32_t piece = 4 * 2048;
            int cc = 0;
            for (int it = 0; it < niter && !*abort_flag; ++it) {
                int z, m0, nt;
                tile_of(it, z, m0, nt);
                const bool skip = vgated(z);
                for (int ch = 0; ch < nck; ++ch, ++cc) {
                    const int sl = cc % g.ering;
                    // one thread: its waits suspend on the barrier (as in tc_fp32p.cu)
                    if (cc >= g.ering && !mbar_wait_timed(&eempty[sl], (uint32_t)(((cc / g.ering) - 1) & 1))) { fail(); break; }
                    unsigned char *dst = reinterpret_cast<unsigned char *>(stage) + (size_t)sl * g.echunk;
                    if (skip || (!g.accumulate && !dg)) {
                        mbar_arrive(&efull[sl]);
                        continue;
                    }
                    mbar_arrive_expect_tx(&efull[sl], (g.accumulate ? piece : 0u) + (dg ? 2 * piece : 0u));
                    const int n0 = nt * NT + ch * 8;
                    #pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int m = m0 + 32 * j;
                        const int c0 = m % Mi32, c2 = m / Mi32;
                        if (g.accumulate) tma_load_4d(dst + j * 2048, &tmC, c0, n0, c2, z, &efull[sl]);
                        if (dg) {
                            tma_load_3d(dst + piece + j * 2048, &tmV, c0, n0, c2, &efull[sl]);
                            tma_load_4d(dst + 2 * piece + j * 2048, &tmX, c0, n0, c2, z, &efull[sl]);
                        }
                    }
                }
            }
            for (int q = cc - g.ering < 0 ? 0 : cc - g.ering; q < cc; ++q)
                mbar_wait_timed(&efull[q % g.ering], (uint32_t)((q / g.ering) & 1), 200000000ull);
        }
        __syncwarp();
    } else if (warp == kQLoadWarp) {
        // ------------------------------------------------------ load lane --
        if (lane == 0) {
            int pit = 0, pks = 0, pz = 0, pm0 = 0, pnt = 0;
            bool pskip = false;
            if (nsteps > 0) { tile_of(0, pz, pm0, pnt); pskip = vgated(pz); }
            int prod = 0;
            for (; prod < nsteps && !*abort_flag; ++prod) {
                const int sl = prod % kQSlots;
                if (prod >= kQSlots && !mbar_wait_timed(&empty[sl], (uint32_t)(((prod / kQSlots) - 1) & 1))) { fail(); break; }
                unsigned char *dst = slots + sl * kQSlot;
                if (pskip) {
                    mbar_arrive(&full[sl]);
                } else {
                    mbar_arrive_expect_tx(&full[sl], (uint32_t)(kQSlabA + bstep));
                    if (kmajor) {
                        tma_load_3d(dst, &tmA, pks * 16, pm0, pz, &full[sl]);
                    } else {
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int m = pm0 + 32 * j;
                            tma_load_4d(dst + j * 4096, &tmA, m % Mi32, pks * 16, m / Mi32, pz, &full[sl]);
                        }
                    }
                    bulk_g2s(dst + kQSlabA, g.bdig + ((size_t)pnt * KS + pks) * kQDig * NT * 16, (uint32_t)bstep,
                             &full[sl]);
                }
                if (++pks == KS) {
                    pks = 0;
                    if (++pit < niter) { tile_of(pit, pz, pm0, pnt); pskip = vgated(pz); }
                }
            }
            for (int q = prod - kQSlots < 0 ? 0 : prod - kQSlots; q < prod; ++q)
                mbar_wait_timed(&full[q % kQSlots], (uint32_t)((q / kQSlots) & 1), 200000000ull);
        }
        __syncwarp();
    } else if (warp == kQMmaWarp) {
        // -------------------------------------------------------- MMA lane --
        if (lane == 0) {
            // group accumulator g at TMEM column g NT, the B digit planes of a step
            // consecutive: one MMA of A_s with the planes t .. t+c-1 (N = c NT <= 256)
            // writes the groups s+t .. s+t+c-1 at once
            const int per = (256 / NT) < kQDig ? 256 / NT : kQDig;
            int q = 0, it = 0, fs = 0, p = 0;
            uint32_t fph = 0, pph = 0;
            for (; it < niter && !*abort_flag; ++it) {
                if (it >= 1 && !mbar_wait(accempty, (uint32_t)((it - 1) & 1))) { fail(); break; }
                for (int ks = 0; ks < KS; ++ks, ++q) {
                    if (!mbar_wait(&pfull[p], pph) || !mbar_wait(&full[fs], fph)) { fail(); break; }
                    fence_after();
                    const unsigned char *Ab = planes + p * kQPlane;
                    const unsigned char *Bb = slots + fs * kQSlot + kQSlabA;
                    #pragma unroll 1
                    for (int s = 0; s < kQDig; ++s) {
                        const uint64_t ad = smem_desc(smem_addr(Ab + s * (kQM * 32)), 128, 256);
                        #pragma unroll 1
                        for (int t = 0; t + s < kQDig; t += per) {
                            const int cnt = (kQDig - s - t) < per ? (kQDig - s - t) : per;
                            const uint64_t bd = smem_desc(smem_addr(Bb + t * (NT * 32)), 128, 256);
                            tc_mma(tbase + (uint32_t)((s + t) * NT), ad, bd, idesc_bf16(cnt * NT),
                                   (ks > 0 || s > 0) ? 1u : 0u);
                        }
                    }
                    tc_commit(&pfree[p]);
                    tc_commit(&empty[fs]);
                    if (++fs == kQSlots) { fs = 0; fph ^= 1u; }
                    if (++p == kQPlanes) { p = 0; pph ^= 1u; }
                }
                if (*abort_flag) break;
                tc_commit(accfull);
            }
            tc_commit(drain);
            mbar_wait_timed(drain, 0, 200000000ull);
        }
        __syncwarp();
    } else {
        // -------------------------------------------------------- epilogue --
        const int qd = warp & 3;                 // TMEM lanes 32 qd .. 32 qd + 31
        const int ew = warp - kQConv / 32;
        const int hc = ew >> 2;                  // this warp's half of the N tile
        double *stg0 = stage + ew * 2 * kQStage;
        const uint32_t lane_base = (uint32_t)(qd * 32) << 16;
        const int half = NT / 2;                 // a multiple of 8
        int nstore = 0;
        for (int it = 0; it < niter; ++it) {
            int z, m0, nt;
            tile_of(it, z, m0, nt);
            bool ok = !*abort_flag;
            if (ok && !mbar_wait_sleep(accfull, (uint32_t)(it & 1), 256)) { fail(); ok = false; }
            ok = __all_sync(0xffffffffu, ok);
            fence_after();
            if (ok && !vgated(z)) {
                const int ex = (m0 + qd * 32 + lane < g.M) ? g.rexp[(i64)z * g.M + m0 + qd * 32 + lane] : 0;
                const double shift = g.shiftv ? g.shiftv[z] : g.shift;
                const double *Vd = g.diagV;
                const double *Xd = g.diagX + (i64)z * g.dx_sz;
                double *C = g.C + (i64)z * g.c_sz;
                const int r = qd * 32 + lane;
                const int m = m0 + r;
                const bool mval = m < g.M;
                const i64 moff = mval ? rowoff(m) : 0;
                const double rs = (g.rowscale && mval) ? g.rowscale[m % Mi32] : 1.0;
                const int sw = (lane >> 1) & 3;
                const bool rows_in = m0 + qd * 32 < g.M;
                // exact group sums -> 64-bit integer -> FP64, times 2^e_n (an
                // exponent add on the bits) and the row's scale
                // T 2^(e_x + e_n - 49), |T| < 2^60, rounded to nearest even and
                // assembled from integer operations (the FP64 pipe is the scarce
                // one); then the row's scale when it is not 1
                const bool unit = (g.alpha * rs == 1.0);
                auto recombine = [&](const float *gq, int n) -> double {
                    // three 32-bit partial sums (each below 2^31), two 64-bit steps
                    const int hi = (__float2int_rn(gq[0]) << 7) + __float2int_rn(gq[1]);
                    const int md = (__float2int_rn(gq[2]) << 7) + __float2int_rn(gq[3]);
                    const int lo = (__float2int_rn(gq[4]) << 7) + __float2int_rn(gq[5]) + (__float2int_rn(gq[6]) >> 7);
                    const long long T = ((long long)hi << 28) + ((long long)md << 14) + lo;
                    if (T == 0 || n >= g.N) return 0.0;
                    const unsigned long long sgn = (unsigned long long)T & 0x8000000000000000ULL;
                    const unsigned long long a = T < 0 ? (unsigned long long)(-T) : (unsigned long long)T;
                    const int lz = __clzll((long long)a);
                    const unsigned long long top = a << lz;              // leading one at bit 63
                    unsigned long long mant = top >> 11;                   // 53 bits
                    const unsigned long long low = top & 0x7FFULL;
                    if (low > 0x400ULL || (low == 0x400ULL && (mant & 1ULL))) ++mant;
                    int ef = 1023 + 63 - lz + ex - 49 + g.bexp[n];
                    if (mant >> 53) { mant >>= 1; ++ef; }
                    double val;
                    if (ef > 0 && ef < 2047)
                        val = __longlong_as_double((long long)(sgn | ((unsigned long long)ef << 52) |
                                                               (mant & 0x000FFFFFFFFFFFFFULL)));
                    else
                        val = ldexp((double)T, ex - 49 + g.bexp[n]);   // outside the normal range
                    return unit ? val : val * (g.alpha * rs);
                };
                if (g.tstore) {
                    // rows along n, nothing to add: 32 x 8 blocks through a
                    // 64-byte-swizzled stage, one TMA store each (rows and
                    // columns past the level's last are clipped)
                    for (int c0 = hc * half; c0 < hc * half + half; c0 += 8) {
                        float gv[kQDig][8];
                        #pragma unroll
                        for (int gq = 0; gq < kQDig; ++gq)
                            tmem_ld8(tbase + lane_base + (uint32_t)(gq * NT + c0), gv[gq]);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        double *stg = stg0 + (nstore & 1) * kQStage;
                        if (nstore >= 2) {
                            if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                            __syncwarp();
                        }
                        #pragma unroll
                        for (int c2 = 0; c2 < 4; ++c2) {
                            float g0[kQDig], g1[kQDig];
                            #pragma unroll
                            for (int gq = 0; gq < kQDig; ++gq) { g0[gq] = gv[gq][2 * c2]; g1[gq] = gv[gq][2 * c2 + 1]; }
                            const int n = nt * NT + c0 + 2 * c2;
                            *reinterpret_cast<double2 *>(stg + lane * 8 + 2 * (c2 ^ sw)) =
                                make_double2(recombine(g0, n), recombine(g1, n + 1));
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0 && rows_in) {
                            tma_store_3d(&tmC, stg, nt * NT + c0, m0 + qd * 32, z);
                            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                        }
                        ++nstore;
                    }
                } else if (g.ering > 0) {
                    // points fastest: per 8-column chunk (this warp's: every
                    // other one), the operands wait in the ring as [8 n][32
                    // points] per quarter; the result overwrites the output's box,
                    // which one TMA copy stores (points past the vector's last
                    // are clipped); the slot is released once the copy read it
                    const int nck = NT / 8;
                    for (int ch = hc; ch < nck; ch += 2) {
                        const int cc = it * nck + ch;
                        const int sl = cc % g.ering;
                        const int c0 = ch * 8;
                        float gv[kQDig][8];
                        #pragma unroll
                        for (int gq = 0; gq < kQDig; ++gq)
                            tmem_ld8(tbase + lane_base + (uint32_t)(gq * NT + c0), gv[gq]);
                        bool eok = !*abort_flag && mbar_wait(&efull[sl], (uint32_t)((cc / g.ering) & 1));
                        eok = __all_sync(0xffffffffu, eok);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        if (!eok) { fail(); break; }
                        double *cb = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(stage) +
                                                                (size_t)sl * g.echunk) + qd * 256;
                        #pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int n = nt * NT + c0 + j;
                            const int idx = j * 32 + lane;
                            float gj[kQDig];
                            #pragma unroll
                            for (int gq = 0; gq < kQDig; ++gq) gj[gq] = gv[gq][j];
                            double o = recombine(gj, n);
                            if (Vd) o = fma(g.alpha * (cb[1024 + idx] - shift), cb[2048 + idx], o);
                            if (g.accumulate) o += cb[idx];
                            cb[idx] = o;
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            if (rows_in) {
                                const int mq = m0 + qd * 32;
                                tma_store_4d(&tmC, cb, mq % Mi32, nt * NT + c0, mq / Mi32, z);
                                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                                ++nstore;
                            }
                            mbar_arrive(&eempty[sl]);
                        }
                        __syncwarp();
                    }
                } else {
                    // rows along n with a diagonal term or an output to add (rare):
                    // direct loads and stores, 4 columns at a time
                    for (int c0 = hc * half; c0 < hc * half + half; c0 += 4) {
                        float gv[kQDig][4];
                        #pragma unroll
                        for (int gq = 0; gq < kQDig; ++gq)
                            tmem_ld4(tbase + lane_base + (uint32_t)(gq * NT + c0), gv[gq]);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                        if (!mval) continue;
                        #pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int n = nt * NT + c0 + j;
                            if (n >= g.N) break;
                            float gj[kQDig];
                            #pragma unroll
                            for (int gq = 0; gq < kQDig; ++gq) gj[gq] = gv[gq][j];
                            const i64 pp = moff + (i64)n * g.c_sn;
                            double o = recombine(gj, n);
                            if (Vd) o = fma(g.alpha * (Vd[pp] - shift), Xd[pp], o);
                            if (g.accumulate) o += C[pp];
                            C[pp] = o;
                        }
                    }
                }
            } else if (ok && g.ering > 0) {
                // a stopped vector: its ring chunks are released unread
                const int nck = NT / 8;
                for (int ch = hc; ch < nck; ch += 2) {
                    const int cc = it * nck + ch;
                    const int sl = cc % g.ering;
                    if (lane == 0) {
                        if (mbar_wait(&efull[sl], (uint32_t)((cc / g.ering) & 1))) mbar_arrive(&eempty[sl]);
                        else fail();
                    }
                    __syncwarp();
                }
            }
            fence_before();
            mbar_arrive(accempty);
        }
        if (lane == 0 && nstore > 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }

    fence_before();
    __syncthreads();
    if (warp == kQMmaWarp)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(512) : "memory");
}

// Binary exponent of the largest |x| of every row of a level, for rows of
// all vectors (out[z M + m]): rows along k (a_sk == 1) one warp per row,
// otherwise 32 consecutive rows (consecutive points) per block, each of its
// kRexpSlices warps taking every kRexpSlices-th k, the slices' maxima
// combined in shared memory (enough blocks for one vector to fill the GPU).
static constexpr int kRexpSlices = 8;
__global__ void rowexp_kernel(const double *__restrict__ X, i64 N, int M, int K, i64 Mi, i64 s1, i64 s2, i64 a_sk,
                              int nvec, int *__restrict__ out, const int *gate, const int *vgate, int vgstride)
{
    if (gate && *gate) return;
    const i64 rows = (i64)M * nvec;
    if (a_sk != 1) {
        __shared__ unsigned long long red[kRexpSlices][32];
        const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
        const i64 t = blockIdx.x * (i64)32 + lane;
        unsigned long long mx = 0;
        bool on = t < rows;
        int z = 0, m = 0;
        if (on) {
            z = (int)(t / M);
            m = (int)(t - (i64)z * M);
            on = !(vgate && vgate[(i64)z * vgstride]);
        }
        if (on) {
            const double *x = X + (i64)z * N + (i64)(m % Mi) * s1 + (i64)(m / Mi) * s2;
            for (int k = slice; k < K; k += kRexpSlices)
                mx = max(mx, (unsigned long long)__double_as_longlong(fabs(x[(i64)k * a_sk])));
        }
        red[slice][lane] = mx;
        __syncthreads();
        if (slice == 0 && on) {
            #pragma unroll
            for (int q = 1; q < kRexpSlices; ++q) mx = max(mx, red[q][lane]);
            out[t] = q_exp(mx);
        }
        return;
    }
    {
        const i64 w = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
        const int lane = threadIdx.x & 31;
        if (w >= rows) return;
        const int z = (int)(w / M), m = (int)(w - (i64)z * M);
        if (vgate && vgate[(i64)z * vgstride]) return;
        const double *x = X + (i64)z * N + (i64)(m % Mi) * s1 + (i64)(m / Mi) * s2;
        unsigned long long mx = 0;
        for (int k = lane; k < K; k += 32) mx = max(mx, (unsigned long long)__double_as_longlong(fabs(x[k])));
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) out[w] = q_exp(mx);
    }
}

// ------------------------------------------------------------------ host --

// Row exponents of every level the persistent kernel takes, for up to
// kQRexpVec vectors (one region per level).
static constexpr int kQRexpVec = 32;

int tc64p_prepare(scalit_ctx *c)
{
    const Layout &L = c->L;
    if (c->rexp) { cudaFree(c->rexp); c->rexp = nullptr; }
    i64 total = 0;
    for (int l = 0; l < L.nlev; ++l) {
        c->rexp_off[l] = total;
        total += (L.N / L.n[l]) * kQRexpVec;
    }
    SC_CUDA(cudaMalloc(&c->rexp, sizeof(int) * (size_t)total));
    return 0;
}

// The persistent FP64 kernel applies to level l when the digit engine holds a
// plan for it (N tile <= 64 columns, K <= 160) and the operand's rows allow
// the tensor copies: rows along k of an even length, or points fastest in
// blocks of a multiple of 32.
bool tc64p_usable(const scalit_ctx *c, int l)
{
    const Layout &L = c->L;
    if (L.ndvr && l == L.nlev - 1) return false;
    const TcLevelData &t = c->tc[l];
    if (!t.usable || t.NT > kQNTMax || t.NT % 16 || !c->rexp) return false;
    const int nout = L.n[l];
    const i64 nin = L.dim[l];
    if (L.N % 2 || nout % 2 || nout > 160) return false;
    if (nin > 1 && nin % 32) return false;
    return true;
}

int tc64p_vectors_max() { return kQRexpVec; }

// The row exponents of level l's rows for nvec vectors of X.
int tc64p_rowexp(const scalit_ctx *c, int l, const double *X, int nvec, const int *gate, cudaStream_t s,
                 const int *vgate, int vstride)
{
    const Layout &L = c->L;
    if (nvec > kQRexpVec) { set_error("more than %d vectors in one FP64 tensor-core launch", kQRexpVec); return SCALIT_EINVAL; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l];
    const i64 M = nin == 1 ? blk : nin * blk;
    const i64 Mi = nin == 1 ? blk : nin, s1 = nin == 1 ? nout : 1, s2 = nin == 1 ? 0 : nin * nout;
    const i64 a_sk = nin == 1 ? 1 : nin;
    const i64 rows = M * nvec;
    // rows along k: a warp per row; points fastest: 32 rows per block of
    // 32 x kRexpSlices threads
    const i64 blocks = a_sk == 1 ? (rows * 32 + 255) / 256 : (rows + 31) / 32;
    rowexp_kernel<<<(unsigned)blocks, a_sk == 1 ? 256 : 32 * kRexpSlices, 0, s>>>(
        X, L.N, (int)M, nout, Mi, s1, s2, a_sk, nvec, c->rexp + c->rexp_off[l], gate, vgate, vstride);
    SC_CHECK_LAUNCH();
    return 0;
}

int tc64p_level_apply(const scalit_ctx *c, int l, const double *X, double *Y, int accumulate, const double *diagV,
                      double shift, double alpha, const int *gate, cudaStream_t s, int nvec, const double *shiftv,
                      const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const TcLevelData &t = c->tc[l];
    if (!tc64p_usable(c, l)) { set_error("level %d has no persistent FP64 tensor-core plan", l + 1); return SCALIT_EUNSUP; }
    if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Y) & 15)) {
        set_error("persistent FP64 tensor-core operands not 16-byte aligned");
        return SCALIT_EINVAL;
    }
    if (nvec > kQRexpVec) { set_error("more than %d vectors in one persistent launch", kQRexpVec); return SCALIT_EINVAL; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    Tc64pArgs g{};
    g.N = nout; g.K = nout; g.KS = t.KS; g.NT = t.NT; g.ntn = t.ntiles;
    if (nin == 1) {
        g.M = (int)blk; g.Mi = blk; g.s1 = nout; g.s2 = 0; g.a_sk = 1; g.c_sn = 1;
        g.rowscale = nullptr;
    } else {
        const i64 M = nin * blk;
        if (M > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
        g.M = (int)M; g.Mi = nin; g.s1 = 1; g.s2 = nin * nout; g.a_sk = nin; g.c_sn = nin;
        g.rowscale = L.dep[l] ? c->DEP + L.deps[l] : nullptr;
    }
    g.mtiles = (g.M + kQM - 1) / kQM;
    const i64 tiles = (i64)g.mtiles * g.ntn * nvec;
    if (tiles > 2147483647LL) { set_error("level %d: too many tiles", l + 1); return SCALIT_EINVAL; }
    g.tiles = (int)tiles;
    g.C = Y; g.c_sz = N;
    g.accumulate = accumulate; g.alpha = alpha;
    g.diagV = diagV; g.diagX = X; g.dx_sz = N; g.shift = shift; g.shiftv = shiftv;
    g.vgate = vgate; g.vgate_stride = vstride;
    g.gate = gate; g.err = c->tc_err;
    g.bdig = t.dig;
    g.bexp = t.exps;
    g.rexp = c->rexp + c->rexp_off[l];
    g.tstore = (g.c_sn == 1 && !accumulate && !diagV) ? 1 : 0;

    // the grid operand: [vector][row][k] boxes of 16 k x 128 rows (128-byte
    // swizzle) or [vector][block][k][point] boxes of 32 points x 16 k; the
    // level-1 output for TMA stores: [vector][row][n] boxes of 8 n x 32 rows
    CUtensorMap tmA, tmC, tmV, tmX;
    int rc;
    if (nin == 1) {
        const cuuint64_t dims[3] = {(cuuint64_t)nout, (cuuint64_t)blk, (cuuint64_t)nvec};
        const cuuint64_t str[2] = {(cuuint64_t)nout * 8, (cuuint64_t)N * 8};
        const cuuint32_t box[3] = {16, kQM, 1};
        rc = tma_encode(&tmA, X, true, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B);
        if (!rc && g.tstore) {
            const cuuint32_t boxc[3] = {8, 32, 1};
            rc = tma_encode(&tmC, Y, true, 3, dims, str, boxc, CU_TENSOR_MAP_SWIZZLE_64B);
        }
    } else {
        const cuuint64_t dims[4] = {(cuuint64_t)nin, (cuuint64_t)nout, (cuuint64_t)blk, (cuuint64_t)nvec};
        const cuuint64_t str[3] = {(cuuint64_t)nin * 8, (cuuint64_t)nin * nout * 8, (cuuint64_t)N * 8};
        const cuuint32_t box[4] = {32, 16, 1, 1};
        rc = tma_encode(&tmA, X, true, 4, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE);
        // the epilogue's operands in 32-point x 8-column boxes: the output (loaded
        // to accumulate, stored back), X and V (without the vector dimension)
        const cuuint32_t boxe[4] = {32, 8, 1, 1};
        if (!rc) rc = tma_encode(&tmC, Y, true, 4, dims, str, boxe, CU_TENSOR_MAP_SWIZZLE_NONE);
        if (!rc && diagV) rc = tma_encode(&tmX, X, true, 4, dims, str, boxe, CU_TENSOR_MAP_SWIZZLE_NONE);
        if (!rc && diagV) rc = tma_encode(&tmV, diagV, true, 3, dims, str, boxe, CU_TENSOR_MAP_SWIZZLE_NONE);
        g.ering = q_ring(diagV != nullptr, &g.echunk);
        if (g.ering < 2) { set_error("level %d: no room for the epilogue ring", l + 1); return SCALIT_EUNSUP; }
    }
    if (rc) return rc;
    if (nin == 1 && !g.tstore) tmC = tmA;
    if (!(nin > 1 && diagV)) { tmV = tmA; tmX = tmA; }

    static int sms = 0, configured = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        SC_CUDA(cudaFuncSetAttribute(tc64p_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kQMaxSmem));
        configured = dev;
    }
    const int grid = (int)(tiles < sms ? tiles : sms);
    const size_t smem = q_smem_bytes((size_t)g.ering * g.echunk);
    if (smem > (size_t)kQMaxSmem) { set_error("persistent FP64 tile too large"); return SCALIT_EUNSUP; }
    tc64p_level_kernel<<<grid, kQThreads, smem, s>>>(g, tmA, tmC, tmV, tmX);
    SC_CHECK_LAUNCH();
    return 0;
}

}  // namespace sc
