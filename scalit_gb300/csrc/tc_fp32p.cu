// Persistent FP32 level products of H*X on the tcgen05 tensor cores.
//
// One CTA per SM walks a strided sequence of 128-row tiles of the grid
// operand (all vectors of the launch), with the level matrix held in shared
// memory for the whole launch.  Three groups of warps run a pipeline:
//
//   converters (warps 0-7)  load 16-wide K slabs of the FP32 grid operand into
//                           a ring of shared-memory slots (16-byte cp.async,
//                           kPDepth slabs in flight), cut each slab into its
//                           hi/lo planes (K-major canonical layout) in a second
//                           ring, and arrive on the plane's mbarrier;
//   MMA warp (warp 16)      issues the three products of every K step into one
//                           of two TMEM accumulators and commits them to the
//                           plane's "free" barrier and, after a tile's last K
//                           step, to the accumulator's "full" barrier;
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
// epilogue.  Rows contiguous along k (level 1, a_sk == 1) give outputs
// contiguous along n: each epilogue warp stages a 32 x 16 block in shared
// memory and stores it as whole 64-byte row pieces.  Otherwise (a_sk > 1)
// a warp's 32 TMEM lanes are 32 consecutive grid points of one column and
// its loads and stores are coalesced as they come.
//
// Every mbarrier wait is bounded; an expired wait raises a shared abort flag
// after which no role waits again, the converters keep meeting at their
// named barrier, the MMA warp stops issuing, the error word is set and the
// CTA frees its TMEM and returns.
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace sc {

static constexpr int kPM = 128;                       // grid rows per tile = TMEM lanes
static constexpr int kPConv = 256;                    // converter threads
static constexpr int kPEpiWarps = 8;                  // two per TMEM lane quarter
static constexpr int kPThreads = kPConv + 32 * kPEpiWarps + 32;
static constexpr int kPMmaWarp = kPConv / 32 + kPEpiWarps;
static constexpr int kPDepth = 6;                     // K slabs in flight
static constexpr int kPSlots = kPDepth + 2;           // FP32 slab slots
static constexpr int kPPlanes = 4;                    // hi/lo plane slots
static constexpr int kPSlab = kPM * 16 * 4;           // one FP32 slab: 8 KB
static constexpr int kPPlane = kPM * 16 * 2 * 2;      // hi + lo planes: 8 KB
static constexpr int kPStage = 32 * 16;               // floats per epilogue warp stage
static constexpr int kPAccCols = 256;                 // TMEM columns per accumulator
static constexpr int kPMaxSmem = 227 * 1024;
static constexpr int kPMaxVec = 4096;                 // vectors per launch (scale slots)

struct Tc32pArgs {
    int M, K, KS, NT, N;       // rows per vector, contraction, K steps, tile columns, output columns
    int mtiles, tiles;         // M tiles per vector, M tiles x vectors
    i64 Mi, s1, s2, a_sk, c_sn;
    const float *A; i64 a_sz;
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
};

static size_t p_smem_bytes(int NT, int KS)
{
    return (size_t)KS * 2 * NT * 32 + (size_t)kPSlots * kPSlab + (size_t)kPPlanes * kPPlane +
           (size_t)kPEpiWarps * kPStage * 4 + 256 * 4 + (2 * kPPlanes + 5) * 8 + 16;
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

template <bool F16>
__global__ void __launch_bounds__(kPThreads, 1)
tc32p_level_kernel(Tc32pArgs g)
{
    if (g.gate && *g.gate) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int NT = g.NT, KS = g.KS;
    const int bstep = 2 * NT * 32;                              // bytes of one K step of B (hi + lo)
    unsigned char *Bs = smem;
    unsigned char *slots = Bs + (size_t)KS * bstep;
    unsigned char *planes = slots + kPSlots * kPSlab;
    float *stage = reinterpret_cast<float *>(planes + kPPlanes * kPPlane);
    float *binv_s = stage + kPEpiWarps * kPStage;
    uint64_t *pfull = reinterpret_cast<uint64_t *>(binv_s + 256);
    uint64_t *pfree = pfull + kPPlanes;
    uint64_t *accfull = pfree + kPPlanes;
    uint64_t *accempty = accfull + 2;
    uint64_t *bready = accempty + 2;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bready + 1);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bready + 1) + 1;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int G = gridDim.x;
    const int niter = (g.tiles - (int)blockIdx.x + G - 1) / G;  // tiles of this CTA
    const bool kmajor = (g.a_sk == 1);
    const int Mi32 = (int)g.Mi;
    auto rowoff = [&](int m) -> i64 {
        const int mq = m / Mi32;
        return (i64)(m - mq * Mi32) * g.s1 + (i64)mq * g.s2;
    };
    auto vgated = [&](int z) -> bool { return g.vgate && g.vgate[(i64)z * g.vgate_stride]; };

    if (tid == 0) {
        for (int i = 0; i < kPPlanes; ++i) { mbar_init(&pfull[i], kPConv); mbar_init(&pfree[i], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&accfull[b], 1); mbar_init(&accempty[b], 32 * kPEpiWarps); }
        mbar_init(bready, 1);
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

    if (warp < 8) {
        // ------------------------------------------------------ converters --
        const int nsteps = niter * KS;
        // Load cursor: the tile and K step of the next slab to request, this
        // thread's two 16-byte pieces (source bases at k = 0, validity) and
        // their fixed destinations in a slot; advanced one step per call.
        int ci = 0, cks = 0;
        const float *cbase[2];
        bool cval[2];
        uint32_t coff[2];
        int ck[2];                                  // the piece's own k offset within a slab
        #pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int e = tid + r * kPConv;
            if (kmajor) {
                const int row = e >> 2, c = e & 3;
                coff[r] = row * 64 + 16 * (c ^ ((row >> 1) & 3));
                ck[r] = 4 * c;
            } else {
                const int kk = e >> 5, c = e & 31;
                coff[r] = kk * 512 + c * 16;
                ck[r] = kk;
            }
        }
        auto tile_bases = [&](int it) {
            const int tau = (int)blockIdx.x + it * G;
            const int z = tau / g.mtiles, m0 = (tau - z * g.mtiles) * kPM;
            const bool skip = vgated(z);
            const float *A = g.A + (i64)z * g.a_sz;
            #pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int e = tid + r * kPConv;
                const int m = kmajor ? m0 + (e >> 2) : m0 + 4 * (e & 31);
                cval[r] = !skip && m < g.M;
                cbase[r] = cval[r] ? A + rowoff(m) + (kmajor ? (i64)ck[r] : (i64)ck[r] * g.a_sk) : g.A;
            }
        };
        if (nsteps > 0) tile_bases(0);
        int qi = 0;                                 // steps requested so far
        auto issue = [&]() {
            if (qi < nsteps) {
                const uint32_t st = smem_addr(slots + (qi % kPSlots) * kPSlab);
                const int k0 = cks * 16;
                #pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const bool v = cval[r] && k0 + ck[r] < g.K;
                    const float *src = v ? cbase[r] + (kmajor ? (i64)k0 : (i64)k0 * g.a_sk) : g.A;
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                                 :: "r"(st + coff[r]), "l"(src), "r"(v ? 16u : 0u) : "memory");
                }
                ++qi;
                if (++cks == KS) {
                    cks = 0;
                    if (++ci < niter) tile_bases(ci);
                }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        for (int q = 0; q < kPDepth; ++q) issue();
        const int row = tid & (kPM - 1), h = tid >> 7;
        const int poff = (row >> 3) * 256 + h * 128 + (row & 7) * 16;
        const int sw = (row >> 1) & 3;
        int ks = 0, it = 0;
        float xs = 1.0f;
        if (F16 && nsteps > 0) xs = p_pow2(p_scale_exp(g.xmax[(int)blockIdx.x / g.mtiles]));
        int slot = 0, p = 0;
        uint32_t pphase = 0;
        // Two K steps per pass: one wait, one barrier and one fence for both,
        // so their fixed latencies are paid once per pair.  The two slots
        // refilled after the barrier held the previous pass's steps, which
        // every converter has finished reading once it reaches the barrier.
        for (int q = 0; q < nsteps; q += 2) {
            asm volatile("cp.async.wait_group %0;" :: "n"(kPDepth - 2) : "memory");
            asm volatile("bar.sync 1, %0;" :: "n"(kPConv) : "memory");
            const int nu = (q + 1 < nsteps) ? 2 : 1;
            uint32_t hw[2][4], lw[2][4];
            #pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (u >= nu) break;
                const unsigned char *st = slots + (slot + u < kPSlots ? slot + u : slot + u - kPSlots) * kPSlab;
                float x[8];
                if (kmajor) {
                    const float4 a = *reinterpret_cast<const float4 *>(st + row * 64 + 16 * ((2 * h) ^ sw));
                    const float4 b = *reinterpret_cast<const float4 *>(st + row * 64 + 16 * ((2 * h + 1) ^ sw));
                    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
                    x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
                } else {
                    const float *sf = reinterpret_cast<const float *>(st);
                    #pragma unroll
                    for (int j = 0; j < 8; ++j) x[j] = sf[(8 * h + j) * kPM + row];
                }
                #pragma unroll
                for (int j = 0; j < 4; ++j) p_cut2<F16>(x[2 * j], x[2 * j + 1], xs, hw[u][j], lw[u][j]);
                if (++ks == KS) {
                    ks = 0;
                    ++it;
                    if (F16 && it < niter) xs = p_pow2(p_scale_exp(g.xmax[((int)blockIdx.x + it * G) / g.mtiles]));
                }
            }
            issue();
            issue();
            #pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (u >= nu) break;
                if (q + u >= kPPlanes && !*abort_flag) {
                    if (!mbar_wait(&pfree[p], pphase ^ 1u)) {
                        *abort_flag = 1;
                        if (g.err) atomicExch(g.err, 5);
                    }
                }
                unsigned char *pl = planes + p * kPPlane;
                *reinterpret_cast<uint4 *>(pl + poff) = make_uint4(hw[u][0], hw[u][1], hw[u][2], hw[u][3]);
                *reinterpret_cast<uint4 *>(pl + kPPlane / 2 + poff) = make_uint4(lw[u][0], lw[u][1], lw[u][2], lw[u][3]);
                if (++p == kPPlanes) { p = 0; pphase ^= 1u; }
            }
            fence_proxy_async_smem();
            {
                int pa = p - nu;
                if (pa < 0) pa += kPPlanes;
                for (int u = 0; u < nu; ++u) {
                    mbar_arrive(&pfull[pa]);
                    if (++pa == kPPlanes) pa = 0;
                }
            }
            slot += 2;
            if (slot >= kPSlots) slot -= kPSlots;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (warp == kPMmaWarp) {
        // -------------------------------------------------------- MMA warp --
        const uint32_t idesc = F16 ? idesc_f16(NT) : idesc_bf16(NT);
        if (!mbar_wait_timed(bready, 0)) { *abort_flag = 1; if (g.err) atomicExch(g.err, 5); }
        int q = 0;
        for (int it = 0; it < niter; ++it) {
            const int b = it & 1;
            if (it >= 2 && !*abort_flag && !mbar_wait_sleep(&accempty[b], (uint32_t)(((it >> 1) - 1) & 1), 64)) {
                *abort_flag = 1;
                if (g.err) atomicExch(g.err, 5);
            }
            fence_after();
            for (int ks = 0; ks < KS; ++ks, ++q) {
                const int p = q % kPPlanes;
                if (!*abort_flag && !mbar_wait_sleep(&pfull[p], (uint32_t)((q / kPPlanes) & 1), 32)) {
                    *abort_flag = 1;
                    if (g.err) atomicExch(g.err, 5);
                }
                fence_after();
                if (lane == 0) {
                    if (!*abort_flag) {
                        const unsigned char *Ab = planes + p * kPPlane;
                        const uint64_t a_hi = smem_desc(smem_addr(Ab), 128, 256);
                        const uint64_t a_lo = smem_desc(smem_addr(Ab + kPPlane / 2), 128, 256);
                        const unsigned char *Bk = Bs + (size_t)ks * bstep;
                        const uint64_t b_hi = smem_desc(smem_addr(Bk), 128, 256);
                        const uint64_t b_lo = smem_desc(smem_addr(Bk + NT * 32), 128, 256);
                        const uint32_t d = tbase + (uint32_t)(b * kPAccCols);
                        tc_mma(d, a_hi, b_hi, idesc, ks > 0 ? 1u : 0u);
                        tc_mma(d, a_hi, b_lo, idesc, 1u);
                        tc_mma(d, a_lo, b_hi, idesc, 1u);
                    }
                    tc_commit(&pfree[p]);
                }
                __syncwarp();
            }
            if (lane == 0) tc_commit(&accfull[b]);
            __syncwarp();
        }
        // every commit has arrived before the TMEM goes (the epilogue waited for
        // the last accumulators; this covers an abort)
        if (niter > 0) {
            mbar_wait_timed(&accfull[(niter - 1) & 1], (uint32_t)(((niter - 1) >> 1) & 1), 200000000ull);
        }
    } else {
        // -------------------------------------------------------- epilogue --
        const int qd = warp & 3;                 // TMEM lanes 32 qd .. 32 qd + 31 (warp % 4)
        const int ew = warp - kPConv / 32;       // 0 .. kPEpiWarps - 1
        const int hc = ew >> 2;                  // this warp's half of the columns
        float *stg = stage + ew * kPStage;
        const int nch = (g.N + 15) / 16;
        const uint32_t lane_base = (uint32_t)(qd * 32) << 16;
        for (int it = 0; it < niter; ++it) {
            const int b = it & 1;
            const int tau = (int)blockIdx.x + it * G;
            const int z = tau / g.mtiles, m0 = (tau - z * g.mtiles) * kPM;
            // the next tile's accumulated output (columns of 128 consecutive
            // grid points) is pulled into L2 while this tile's products run,
            // so the epilogue's loads of it hit L2
            if (g.accumulate && g.c_sn > 1 && it + 1 < niter) {
                const int tn = tau + G;
                const int zn = tn / g.mtiles, mn0 = (tn - zn * g.mtiles) * kPM;
                if (!vgated(zn)) {
                    const int mend = min(mn0 + kPM, g.M);
                    for (int n = ew * 32 + lane; n < g.N; n += 32 * kPEpiWarps) {
                        const float *Cn = g.C + (i64)zn * g.c_sz + (i64)n * g.c_sn;
                        for (int a = mn0; a < mend;) {
                            const int bend = min(mend, (a / Mi32 + 1) * Mi32);
                            prefetch_l2_bulk(Cn + rowoff(a), (uint32_t)(bend - a) * 4u);
                            a = bend;
                        }
                    }
                }
            }
            bool ok = !*abort_flag;
            if (ok && !mbar_wait_sleep(&accfull[b], (uint32_t)((it >> 1) & 1), 256)) {
                *abort_flag = 1;
                if (g.err) atomicExch(g.err, 5);
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
                if (g.c_sn == 1) {
                    // rows contiguous along n: 32 x 16 blocks through the warp's
                    // stage (row scale applied going in, column scale coming out),
                    // stored as 64-byte row pieces; the diagonal term and the
                    // accumulated output, when given, are loaded the same way
                    const int f = lane & 3;
                    const int sw = (lane >> 1) & 3;
                    i64 rbase[4];
                    bool rval[4];
                    #pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int mm = m0 + qd * 32 + 8 * u + (lane >> 2);
                        rval[u] = mm < g.M;
                        rbase[u] = rval[u] ? rowoff(mm) : 0;
                    }
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
                        const bool nval = n < g.N;
                        if (!Vd && !g.accumulate) {
                            #pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const int rr = 8 * u + (lane >> 2);
                                const float4 o = *reinterpret_cast<const float4 *>(stg + rr * 16 + 4 * (f ^ ((rr >> 1) & 3)));
                                if (rval[u] && nval)
                                    *reinterpret_cast<float4 *>(C + rbase[u] + n) =
                                        make_float4(o.x * cs.x, o.y * cs.y, o.z * cs.z, o.w * cs.w);
                            }
                        } else {
                            #pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const int rr = 8 * u + (lane >> 2);
                                const float4 o = *reinterpret_cast<const float4 *>(stg + rr * 16 + 4 * (f ^ ((rr >> 1) & 3)));
                                if (!rval[u] || !nval) continue;
                                const i64 pp = rbase[u] + n;
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
                        }
                        __syncwarp();
                    }
                } else {
                    // a lane owns grid row m; per column the warp's 32 lanes are
                    // 32 consecutive points; groups of 8 columns of this warp's
                    // half, every load of a group (accumulated output, diagonal
                    // term) issued together with the group's TMEM load
                    const bool mval = m < g.M;
                    const i64 moff = mval ? rowoff(m) : 0;
                    for (int ch = hc; ch < nch; ch += 2) {
                        #pragma unroll
                        for (int hf = 0; hf < 2; ++hf) {
                            const int c0 = ch * 16 + 8 * hf;
                            float v[8], cy[8], dv[8], dx[8];
                            tmem_ld8(tbase + lane_base + (uint32_t)(b * kPAccCols + c0), v);
                            #pragma unroll
                            for (int t = 0; t < 8; ++t) {
                                const int n = c0 + t;
                                const bool in = mval && n < g.N;
                                const i64 p = moff + (i64)n * g.c_sn;
                                cy[t] = (in && g.accumulate) ? C[p] : 0.0f;
                                dv[t] = (in && Vd) ? Vd[p] : 0.0f;
                                dx[t] = (in && Vd) ? Xd[p] : 0.0f;
                            }
                            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                            if (!mval) continue;
                            #pragma unroll
                            for (int t = 0; t < 8; ++t) {
                                const int n = c0 + t;
                                if (n >= g.N) break;
                                float out = v[t] * (sc * binv_s[n]) + cy[t];
                                if (Vd) out = fmaf(g.alpha * (dv[t] - shift), dx[t], out);
                                C[moff + (i64)n * g.c_sn] = out;
                            }
                        }
                    }
                }
            } else if (ok) {
                // a stopped vector: the accumulator is released unread
            }
            fence_before();
            mbar_arrive(&accempty[b]);
        }
    }

    // B copies have landed before the shared memory goes (an abort may skip
    // the MMA warp's wait on them)
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

static bool p_fits(int NT, int KS) { return p_smem_bytes(NT, KS) <= (size_t)kPMaxSmem; }

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
        if (NT > 256 || !p_fits(NT, KS)) continue;
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
bool tc32p_usable(const scalit_ctx *c, int l, bool f16)
{
    const Layout &L = c->L;
    if (L.ndvr && l == L.nlev - 1) return false;
    const TcLevelData &t = f16 ? c->tc16[l] : c->tc32[l];
    if (!t.usable || t.ntiles != 1 || !p_fits(t.NT, t.KS)) return false;
    if (f16 && !c->xmax) return false;
    const int nout = L.n[l];
    const i64 nin = L.dim[l], N = L.N;
    if (N % 4 || nout % 4) return false;
    if (nin > 1 && nin % 4) return false;
    return true;
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
    if (!tc32p_usable(c, l, f16)) { set_error("level %d has no persistent tensor-core plan", l + 1); return SCALIT_EUNSUP; }
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
    g.A = X; g.a_sz = N; g.C = Y; g.c_sz = N;
    g.accumulate = accumulate; g.alpha = alpha;
    g.diagV = diagV; g.diagX = X; g.dx_sz = N; g.shift = shift; g.shiftv = shiftv;
    g.vgate = vgate; g.vgate_stride = vstride;
    g.gate = gate; g.err = c->tc_err;
    g.bsplit = reinterpret_cast<const uint4 *>(t.dig);
    g.binv = f16 ? t.cscale : nullptr;
    g.xmax = f16 ? c->xmax : nullptr;

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
    const size_t smem = p_smem_bytes(g.NT, g.KS);
    if (f16) tc32p_level_kernel<true><<<grid, kPThreads, smem, s>>>(g);
    else tc32p_level_kernel<false><<<grid, kPThreads, smem, s>>>(g);
    SC_CHECK_LAUNCH();
    return 0;
}

}  // namespace sc
