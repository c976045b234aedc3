// FP64-accurate level contractions of H*X on the tcgen05 tensor cores.
//
// GB300's FP64 pipe delivers ~1.1 TFLOP/s while its BF16 tensor cores deliver
// ~2 PFLOP/s, so the FP64 level GEMMs  C(m, n) = sum_k A(m, k) B(k, n)
// (A = the grid vector viewed through the level's strides, B(k, n) = H(n, k))
// are computed exactly enough for FP64 from 7-bit integer digits:
//
//   A(m, k) = 2^e_m  sum_{s=0..6} a_s(m, k) 2^-7(s+1),   |a_s| <= 127   (e_m: row exponent)
//   B(k, n) = 2^e_n  sum_{t=0..6} b_t(k, n) 2^-7(t+1),   |b_t| <= 127   (e_n: column exponent)
//   C(m, n) = 2^(e_m+e_n-14) sum_{g=0..6} 2^-7g G_g(m, n),
//   G_g = sum_{s+t=g} sum_k a_s b_t          (28 digit pairs)
//
// Every digit is an integer of at most 7 bits, exact in BF16; a product is at
// most 2^14 and a group of g+1 pairs over K <= 160 stays below 2^24, so the
// FP32 tensor-core accumulation of groups 0..5 is exact (group 6 sits 2^-42
// below group 0, where FP32 rounding is immaterial).  The dropped digits and
// pairs leave a relative error of ~2^-46 of |A||B|.  Each group accumulates
// in its own TMEM accumulator; the epilogue reads them with tcgen05.ld and
// recombines them in FP64.
//
// Structure of a CTA (512 threads, one M tile of 128 grid rows, one N tile):
// four threads own each row.  The FP64 operand streams through shared memory
// in 16-wide K slabs by cp.async (a 3-deep ring), twice: the first pass finds
// each row's exponent, the second cuts every slab into 7 digit planes written
// to shared memory in the K-major canonical layout (8x16-byte core matrices,
// no swizzle); the K step's pre-cut B digit planes are copied next to them;
// thread 0 issues the 28 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) and a
// tcgen05.commit on the buffer's mbarrier.  Two buffers let the cutting of
// step k+1 overlap the MMAs of step k.  Every mbarrier wait is bounded: on
// expiry the kernel records an error, waits (bounded) for its MMAs, frees its
// TMEM and returns.
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sc {

static constexpr int kDigits = 7;
static constexpr int kGroups = 7;
static constexpr int kBM = 128;
static constexpr int kThreadsTC = 512;   // cutting threads: four per grid row
static constexpr int kBlockTC = 544;     // plus one warp that issues the MMAs
static constexpr int kTmemCols = 512;
static constexpr int kStages = 8;                               // FP64 slab ring depth
static constexpr int kSlab = kBM * 17;                          // doubles per slab stage
static constexpr int kAStepBytes = kDigits * kBM * 16 * 2;    // 7 digit planes of 128 x 16 BF16

struct TcArgs {
    int M, N, K, KS, NT;
    i64 Mi, s1, s2, a_sk, c_sn;
    const double *A; i64 a_sz;
    double *C; i64 c_sz;
    const double *rowscale;
    int accumulate;
    double alpha;
    const double *diagV;
    const double *diagX;
    i64 dx_sz;
    double shift;
    const double *shiftv;   // per-vector shifts (vector index z), overriding shift
    const int *vgate;       // per-vector stop flags vgate[z * vgate_stride] (may be null)
    int vgate_stride;
    const int *gate;
    int *err;
    const uint4 *bdig;    // [ntile][ks][digit][NT x 16 BF16, canonical]
    const int *bexp;      // [ntile * NT] column exponents
    // Per-block B (the preconditioner's rotations): every block of Mi grid rows
    // has its own matrix; tpb M tiles cover one block and never straddle two.
    int tpb;              // 0: one B for all rows
    i64 bdig_blk;         // uint4 stride between the blocks' digit planes
    int bexp_blk;         // int stride between the blocks' exponents
};

// Binary exponent e with |x| < 2^e for x != 0 (frexp's exponent), read from the bits.
__device__ __forceinline__ int exp_of(unsigned long long bits)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex) return ex - 1022;
    const unsigned long long m = bits & 0x000FFFFFFFFFFFFFULL;   // subnormal
    return m ? (64 - __clzll(m)) - 1074 : -100000;
}

// 49-bit fixed-point magnitude of |x| 2^(49 - e) (truncated), e >= exponent of x.
__device__ __forceinline__ unsigned long long fixed49(unsigned long long bits, int e)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long m = (bits & 0x000FFFFFFFFFFFFFULL) | (ex ? (1ULL << 52) : 0ULL);
    const int sh = (ex ? ex : 1) - 1075 + 49 - e;   // <= -4
    return (sh <= -64) ? 0ULL : (m >> (-sh));
}

__global__ void __launch_bounds__(kBlockTC, 1)
tc_level_kernel(TcArgs g)
{
    if (g.gate && *g.gate) return;
    if (g.vgate && g.vgate[(i64)blockIdx.z * g.vgate_stride]) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int NT = g.NT, KS = g.KS;
    const int bstep = kDigits * NT * 32;                   // bytes of one K step of B digits
    unsigned char *Abuf = smem;                            // 2 x kAStepBytes
    unsigned char *Bbuf = smem + 2 * kAStepBytes;          // 2 x bstep
    double *slabs = reinterpret_cast<double *>(Bbuf + 2 * bstep);   // kStages x kSlab
    uint64_t *mbar = reinterpret_cast<uint64_t *>(slabs + kStages * kSlab);   // MMAs of a buffer done
    uint64_t *cutb = mbar + 2;                                                  // a buffer's digits cut
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 4);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int ntile = blockIdx.y, z = blockIdx.z;
    // rows [m0, mlim) of this tile; with per-block B the tile stays inside block bsel
    int m0, mlim;
    const uint4 *bdig = g.bdig;
    const int *bexp = g.bexp;
    if (g.tpb > 0) {
        const int bsel = blockIdx.x / g.tpb, lt = blockIdx.x - bsel * g.tpb;
        m0 = bsel * (int)g.Mi + lt * kBM;
        mlim = min(g.M, bsel * (int)g.Mi + (int)g.Mi);
        bdig += (i64)bsel * g.bdig_blk;
        bexp += (i64)bsel * g.bexp_blk;
    } else {
        m0 = blockIdx.x * kBM;
        mlim = g.M;
    }
    const double *A = g.A + (i64)z * g.a_sz;
    double *C = g.C + (i64)z * g.c_sz;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tslot)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init(&cutb[0], kThreadsTC);
        mbar_init(&cutb[1], kThreadsTC);
        mbar_init_fence();
    }

    // BF16 bit patterns of the digits -127..127 (all exact in BF16)
    uint16_t *bf_tab = reinterpret_cast<uint16_t *>(tslot + 4);
    for (int i = tid; i < 255; i += kThreadsTC)
        bf_tab[i] = __bfloat16_as_ushort(__float2bfloat16_rn((float)(i - 127)));
    int *em4 = reinterpret_cast<int *>(bf_tab + 256);       // [4][kBM] partial row exponents

    if (warp == kThreadsTC / 32) {
        // The MMA warp: for every K step, wait until the cutting threads have
        // written the step's digit planes, issue the 28 digit-pair MMAs (one
        // lane) and commit them to the buffer's barrier; the cutting of the
        // next step proceeds meanwhile.
        fence_before();
        __syncthreads();
        fence_after();
        const uint32_t tbase = *tslot;
        // group g at TMEM column g NT and the step's B digit planes consecutive:
        // one product of A_s with the planes t .. t+c-1 (N = c NT <= 256) writes
        // the groups s+t .. s+t+c-1 at once
        const int per = (256 / NT) < kDigits ? 256 / NT : kDigits;
        const int lane = tid & 31;
        for (int ks = 0; ks < KS; ++ks) {
            const int buf = ks & 1;
            if (!mbar_wait(&cutb[buf], (uint32_t)((ks >> 1) & 1))) break;
            fence_after();
            if (lane == 0) {
                const unsigned char *Ab = Abuf + buf * kAStepBytes;
                const unsigned char *Bb = Bbuf + buf * bstep;
                #pragma unroll 1
                for (int s = 0; s < kDigits; ++s) {
                    const uint64_t ad = smem_desc(smem_addr(Ab + s * (kBM * 32)), 128, 256);
                    #pragma unroll 1
                    for (int t = 0; t + s < kGroups; t += per) {
                        const int cnt = (kGroups - s - t) < per ? (kGroups - s - t) : per;
                        const uint64_t bd = smem_desc(smem_addr(Bb + t * (NT * 32)), 128, 256);
                        const uint32_t acc = (ks > 0 || s > 0) ? 1u : 0u;
                        tc_mma(tbase + (uint32_t)((s + t) * NT), ad, bd, idesc_bf16(cnt * NT), acc);
                    }
                }
                tc_commit(&mbar[buf]);
            }
            __syncwarp();
        }
        fence_before();
        __syncthreads();
        return;   // warp 0 frees the TMEM
    }

    // Four threads per grid row: quarter q handles K values 4q..4q+3 of every
    // 16-wide K step.  The cutting threads synchronise among themselves with
    // named barrier 1 (the MMA warp never waits on it).
    const int row = tid & (kBM - 1), q = tid >> 7;
    const int m = m0 + row;
    const bool mvalid = m < mlim;
    const i64 moff = mvalid ? (i64)(m % g.Mi) * g.s1 + (i64)(m / g.Mi) * g.s2 : 0;
    // FP64 operand slabs (16 K values x 128 rows) stream through a kStages ring by
    // cp.async: pass 1 (slabs 0..KS-1) finds the row exponents, pass 2 (slabs
    // KS..2KS-1) cuts the digits.  When K is the contiguous index (a_sk == 1) a
    // slab is stored row by row (stride 17) and consecutive threads copy
    // consecutive K values of a row; otherwise K by K (rows contiguous) and
    // consecutive threads copy consecutive rows.  Both keep the copies coalesced.
    const bool rowc = (g.a_sk == 1);
    i64 lmoff[4];
    bool lvalid[4];
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = rowc ? ((tid >> 4) + 32 * i) : row;
        const int mm = m0 + r;
        lvalid[i] = mm < mlim;
        lmoff[i] = lvalid[i] ? (i64)(mm % g.Mi) * g.s1 + (i64)(mm / g.Mi) * g.s2 : 0;
    }
    auto issue = [&](int t) {
        if (t < 2 * KS) {
            const int ks = t % KS;
            double *st = slabs + (t % kStages) * kSlab;
            #pragma unroll
            for (int i = 0; i < 4; ++i) {
                int r, j;
                if (rowc) { j = tid & 15; r = (tid >> 4) + 32 * i; }
                else { r = row; j = q + 4 * i; }
                const int k = ks * 16 + j;
                double *dst = rowc ? st + r * 17 + j : st + j * kBM + r;
                if (lvalid[i] && k < g.K) {
                    const double *src = A + lmoff[i] + (i64)k * g.a_sk;
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;"
                                 :: "r"(smem_addr(dst)), "l"(src) : "memory");
                } else {
                    *dst = 0.0;
                }
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    auto cut_sync = [&]() { asm volatile("bar.sync 1, %0;" :: "n"(kThreadsTC) : "memory"); };
    auto ready = [&]() {
        asm volatile("cp.async.wait_group %0;" :: "n"(kStages - 2) : "memory");
        cut_sync();
    };
    auto slab_val = [&](const double *st, int j) -> unsigned long long {   // K value j of this row
        return (unsigned long long)__double_as_longlong(rowc ? st[row * 17 + j] : st[j * kBM + row]);
    };
    // With K <= 16 kStages all K slabs fit the ring: they are loaded once, all in
    // flight together, and serve both passes; otherwise they stream twice with
    // kStages - 1 slabs of look-ahead.
    const bool resident = (KS <= kStages);
    if (resident) {
        for (int t = 0; t < KS; ++t) issue(t);
        asm volatile("cp.async.wait_all;" ::: "memory");
        cut_sync();
    } else {
        for (int t = 0; t < kStages - 1; ++t) issue(t);
    }
    int em = -100000;
    for (int t = 0; t < KS; ++t) {
        if (!resident) {
            ready();
            issue(t + kStages - 1);
        }
        const double *st = slabs + (t % kStages) * kSlab;
        #pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const unsigned long long b = slab_val(st, q * 4 + jj);
            if (b << 1) em = max(em, exp_of(b));
        }
    }
    em4[q * kBM + row] = em;
    cut_sync();
    em = max(max(em4[row], em4[kBM + row]), max(em4[2 * kBM + row], em4[3 * kBM + row]));
    if (em < -2000) em = 0;   // an all-zero row

    fence_before();
    __syncthreads();          // with the MMA warp: TMEM address and barriers ready
    fence_after();
    const uint32_t tbase = *tslot;
    bool ok = true;

    for (int ks = 0; ks < KS; ++ks) {
        const int buf = ks & 1;
        if (ks >= 2 && !mbar_wait(&mbar[buf], ((ks - 2) >> 1) & 1)) { ok = false; break; }
        unsigned char *Ab = Abuf + buf * kAStepBytes;
        unsigned char *Bb = Bbuf + buf * bstep;
        const int t = KS + ks;
        if (!resident) {
            ready();
            issue(t + kStages - 1);
        }
        const double *st = slabs + ((resident ? ks : t) % kStages) * kSlab;
        // cut this row's 4 values of the K step (this thread's quarter) into 7
        // digit planes: the digits are the 7-bit fields of the 49-bit fixed-point
        // magnitude, with x's sign
        unsigned long long F[4];
        int sgn[4];
        #pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const unsigned long long b = slab_val(st, q * 4 + jj);
            F[jj] = fixed49(b, em);
            sgn[jj] = (int)(b >> 63);
        }
        const int rowoff = (row >> 3) * 256 + (q >> 1) * 128 + (row & 7) * 16 + (q & 1) * 8;
        #pragma unroll
        for (int s = 0; s < kDigits; ++s) {
            uint32_t w[2];
            #pragma unroll
            for (int jj = 0; jj < 4; jj += 2) {
                const int d0 = (int)((F[jj] >> (42 - 7 * s)) & 127u);
                const int d1 = (int)((F[jj + 1] >> (42 - 7 * s)) & 127u);
                const uint32_t b0 = bf_tab[127 + (sgn[jj] ? -d0 : d0)];
                const uint32_t b1 = bf_tab[127 + (sgn[jj + 1] ? -d1 : d1)];
                w[jj >> 1] = b0 | (b1 << 16);
            }
            *reinterpret_cast<uint2 *>(Ab + s * (kBM * 32) + rowoff) = make_uint2(w[0], w[1]);
        }
        // the K step's B digit planes (pre-cut, already in the canonical layout)
        const uint4 *src = bdig + ((i64)ntile * KS + ks) * (bstep / 16);
        uint4 *dst = reinterpret_cast<uint4 *>(Bb);
        for (int i = tid; i < bstep / 16; i += kThreadsTC) dst[i] = src[i];
        // make the planes visible to the tensor cores, then hand the step over
        fence_proxy_async_smem();
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_addr(&cutb[buf])) : "memory");
    }
    if (ok) ok = mbar_wait(&mbar[(KS - 1) & 1], ((KS - 1) >> 1) & 1);
    asm volatile("cp.async.wait_all;" ::: "memory");   // no copy of this CTA stays in flight
    if (!ok) {
        if (g.err) atomicExch(g.err, 1);
        // give in-flight MMAs a bounded chance to drain before freeing TMEM
        for (int b = 0; b < 2; ++b) mbar_wait(&mbar[b], 0) || mbar_wait(&mbar[b], 1);
    }
    fence_after();

    // Output rows contiguous along n (a level with nin == 1): the recombined
    // values go through shared memory (the A and B digit buffers, free once the
    // last MMA completed; padded stride NT + 1) and each warp then finishes
    // whole rows with the lanes along n, so the diagonal term's loads, the
    // accumulated output and the stores are coalesced instead of every warp
    // store touching 32 rows a row length apart.
    double *stage = reinterpret_cast<double *>(smem);
    const bool staged = (g.c_sn == 1);
    const int sld = NT + 1;

    if (ok) {
        // epilogue: thread tid holds TMEM lane tid = grid row m.  The exact group
        // sums are recombined in 64-bit integers: T = sum_{g<=5} G_g 2^(7(5-g))
        // + floor(G_6 / 2^7) < 2^60, so C = T 2^(e_m + e_n - 49), one conversion.
        const double rs = (g.rowscale && mvalid) ? g.rowscale[m % g.Mi] : 1.0;
        const double sc = g.alpha * rs * ldexp(1.0, em - 49);
        // warp w reads TMEM lanes 32 (w % 4) .. (its rows) and the column quarter w / 4
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int cq = NT / 4;                       // NT is a multiple of 16
        const int cbeg = (warp >> 2) * cq, cend = cbeg + cq;
        for (int c0 = cbeg; c0 < cend; c0 += 4) {
            float gv[kGroups][4];
            #pragma unroll
            for (int gq = 0; gq < kGroups; ++gq) tmem_ld4(tbase + lane_base + (uint32_t)(gq * NT + c0), gv[gq]);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!mvalid) continue;
            // the four outputs with every load (exponents, diagonal,
            // accumulated output) issued before the first store
            double outv[4];
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int n = ntile * NT + c0 + j;
                if (n >= g.N) continue;
                long long T = ((long long)__float2int_rn(gv[kGroups - 1][j])) >> 7;
                #pragma unroll
                for (int gq = kGroups - 2; gq >= 0; --gq)
                    T += (long long)__float2int_rn(gv[gq][j]) << (7 * (kGroups - 2 - gq));
                double val = (double)T;
                if (T != 0)   // times 2^e_n by an exponent add on the bits (no FP64 op)
                    val = __longlong_as_double(__double_as_longlong(val) + ((long long)bexp[n] << 52));
                const i64 p = moff + (i64)n * g.c_sn;
                double out = sc * val;
                if (staged) { outv[j] = out; continue; }
                if (g.diagV) out = fma(g.alpha * (g.diagV[p] - (g.shiftv ? g.shiftv[z] : g.shift)),
                                       g.diagX[p + (i64)z * g.dx_sz], out);
                if (g.accumulate) out += C[p];
                outv[j] = out;
            }
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int n = ntile * NT + c0 + j;
                if (staged) stage[row * sld + c0 + j] = outv[j];
                else if (n < g.N) C[moff + (i64)n * g.c_sn] = outv[j];
            }
        }
    }
    if (staged) {
        // every cutting thread arrives here, whatever its wait results were
        asm volatile("bar.sync 1, %0;" :: "n"(kThreadsTC) : "memory");
        const double shift = g.shiftv ? g.shiftv[z] : g.shift;
        const int lane = tid & 31;
        for (int r = warp; r < kBM && ok; r += kThreadsTC / 32) {
            const int mm = m0 + r;
            if (mm >= mlim) break;
            const i64 ro = (i64)(mm % g.Mi) * g.s1 + (i64)(mm / g.Mi) * g.s2;
            for (int cc = lane; cc < NT; cc += 32) {
                const int n = ntile * NT + cc;
                if (n >= g.N) break;
                const i64 p = ro + n;
                double out = stage[r * sld + cc];
                if (g.diagV) out = fma(g.alpha * (g.diagV[p] - shift), g.diagX[p + (i64)z * g.dx_sz], out);
                if (g.accumulate) out += C[p];
                C[p] = out;
            }
        }
    }
    fence_before();
    __syncthreads();          // with the MMA warp
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(kTmemCols) : "memory");
}

// ------------------------------------------------------------------ host --
// Digit planes of one level matrix: B(k, n) = H(n, k), per column n an
// exponent e_n with |B(k, n)| < 2^e_n, then 7 digits per value.  Packed per
// (N tile, K step, digit) as NT x 16 BF16 in the canonical K-major layout.
static void cut_level_matrix(const double *H, int nout, int NT, int ntiles, int KS, std::vector<uint16_t> &dig,
                             std::vector<int> &exps)
{
    const int KP = KS * 16;
    dig.assign((size_t)ntiles * KS * kDigits * NT * 16, 0);
    exps.assign((size_t)ntiles * NT, 0);
    for (int n = 0; n < nout; ++n) {
        double mx = 0.0;
        for (int k = 0; k < nout; ++k) mx = std::max(mx, std::fabs(H[n + (size_t)nout * k]));
        int e = 0;
        if (mx > 0.0) std::frexp(mx, &e);
        exps[n] = e;
        const int tile = n / NT, nn = n % NT;
        for (int k = 0; k < KP; ++k) {
            double r = (k < nout) ? std::ldexp(H[n + (size_t)nout * k], 7 - e) : 0.0;
            const int ks = k / 16, kk = k % 16;
            for (int t = 0; t < kDigits; ++t) {
                const double d = std::trunc(r);
                r = (r - d) * 128.0;
                const float f = (float)d;
                uint32_t u;
                std::memcpy(&u, &f, 4);
                const uint16_t bits = (uint16_t)(u >> 16);   // exact: |d| <= 127
                const size_t base = (((size_t)tile * KS + ks) * kDigits + t) * (size_t)NT * 16;
                const size_t off = (size_t)(nn >> 3) * 128 + (size_t)(kk >> 3) * 64 + (size_t)(nn & 7) * 8 + (kk & 7);
                dig[base + off] = bits;
            }
        }
    }
}

int tc_prepare(scalit_ctx *c)
{
    const Layout &L = c->L;
    for (int l = 0; l < L.nlev; ++l) {
        TcLevelData &t = c->tc[l];
        if (t.dig) { cudaFree(t.dig); t.dig = nullptr; }
        if (t.exps) { cudaFree(t.exps); t.exps = nullptr; }
        t.usable = 0;
        if (L.ndvr && l == L.nlev - 1) continue;
        const int nout = L.n[l];
        if (nout > 256) continue;   // exactness of the FP32 groups needs K <= 256
        const int NT = std::min(64, (nout + 15) / 16 * 16);
        const int ntiles = (nout + NT - 1) / NT;
        const int KS = (nout + 15) / 16;
        std::vector<double> H(L.h0s[l] >= 0 ? (size_t)nout * nout : 0);
        SC_CUDA(cudaMemcpy(H.data(), c->H0 + L.h0s[l], sizeof(double) * H.size(), cudaMemcpyDeviceToHost));
        std::vector<uint16_t> dig;
        std::vector<int> exps;
        cut_level_matrix(H.data(), nout, NT, ntiles, KS, dig, exps);
        SC_CUDA(cudaMalloc(&t.dig, dig.size() * sizeof(uint16_t)));
        SC_CUDA(cudaMalloc(&t.exps, exps.size() * sizeof(int)));
        SC_CUDA(cudaMemcpy(t.dig, dig.data(), dig.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
        SC_CUDA(cudaMemcpy(t.exps, exps.data(), exps.size() * sizeof(int), cudaMemcpyHostToDevice));
        t.NT = NT;
        t.ntiles = ntiles;
        t.KS = KS;
        t.usable = 1;
    }
    if (!c->tc_err) SC_CUDA(cudaMalloc(&c->tc_err, sizeof(int)));
    SC_CUDA(cudaMemset(c->tc_err, 0, sizeof(int)));
    return 0;
}

// Digit planes of the preconditioner's rotations of level l (VOSB level l:
// blk matrices V_b of n x n).  transpose = 0 plans V_b (VX), 1 plans V_b^T
// (VTX).  One thread per (block, column n of B), B(k, n) = H(n, k) with H = V_b
// or V_b^T; the digits, exponents and layout are those of cut_level_matrix.
__global__ void cut_rot_kernel(int nout, int NT, int ntiles, int KS, int blk, const double *__restrict__ V,
                               int transpose, uint16_t *__restrict__ dig, int *__restrict__ exps)
{
    const i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x;
    if (idx >= (i64)blk * nout) return;
    const int b = (int)(idx / nout), n = (int)(idx - (i64)b * nout);
    const double *Vb = V + (i64)b * nout * nout;
    double mx = 0.0;
    for (int k = 0; k < nout; ++k) {
        const double v = transpose ? Vb[k + (i64)n * nout] : Vb[n + (i64)k * nout];
        mx = fmax(mx, fabs(v));
    }
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    exps[(i64)b * ntiles * NT + n] = e;
    const int tile = n / NT, nn = n % NT;
    for (int k = 0; k < nout; ++k) {
        double r = ldexp(transpose ? Vb[k + (i64)n * nout] : Vb[n + (i64)k * nout], 7 - e);
        const int ks = k / 16, kk = k % 16;
        #pragma unroll
        for (int t = 0; t < kDigits; ++t) {
            const double d = trunc(r);
            r = (r - d) * 128.0;
            const size_t base = ((((size_t)b * ntiles + tile) * KS + ks) * kDigits + t) * (size_t)NT * 16;
            const size_t off = (size_t)(nn >> 3) * 128 + (size_t)(kk >> 3) * 64 + (size_t)(nn & 7) * 8 + (kk & 7);
            dig[base + off] = __bfloat16_as_ushort(__float2bfloat16_rn((float)d));   // |d| <= 127: exact
        }
    }
}

void tc_free_px(scalit_ctx *c)
{
    for (int l = 0; l < SCALIT_FMAX; ++l)
        for (int d = 0; d < 2; ++d) {
            TcLevelData &t = c->pxtc[l][d];
            if (t.dig) cudaFree(t.dig);
            if (t.exps) cudaFree(t.exps);
            t = TcLevelData{};
        }
}

int tc_prepare_px(scalit_ctx *c)
{
    const Layout &L = c->L;
    tc_free_px(c);
    for (int l = 1; l < L.nlev; ++l) {
        const int nout = L.n[l];
        if (nout > 256 || L.dim[l] < 2) continue;   // group exactness needs K <= 256
        const int NT = std::min(64, (nout + 15) / 16 * 16);
        const int ntiles = (nout + NT - 1) / NT;
        const int KS = (nout + 15) / 16;
        const i64 blk = L.blk[l];
        const size_t ndig = (size_t)blk * ntiles * KS * kDigits * NT * 16;
        const size_t nexp = (size_t)blk * ntiles * NT;
        for (int d = 0; d < 2; ++d) {
            TcLevelData &t = c->pxtc[l][d];
            SC_CUDA(cudaMalloc(&t.dig, ndig * sizeof(uint16_t)));
            SC_CUDA(cudaMalloc(&t.exps, nexp * sizeof(int)));
            SC_CUDA(cudaMemsetAsync(t.dig, 0, ndig * sizeof(uint16_t), c->stream));
            SC_CUDA(cudaMemsetAsync(t.exps, 0, nexp * sizeof(int), c->stream));
            const i64 items = blk * nout;
            cut_rot_kernel<<<(int)((items + 127) / 128), 128, 0, c->stream>>>(nout, NT, ntiles, KS, (int)blk,
                                                                               c->VOSB + L.vs[l], d, t.dig, t.exps);
            SC_CHECK_LAUNCH();
            t.NT = NT;
            t.ntiles = ntiles;
            t.KS = KS;
            t.usable = 1;
        }
    }
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

bool tc_px_usable(const scalit_ctx *c, int l)
{
    return c->fp64_mode == SCALIT_FP64_TENSOR && c->pxtc[l][0].usable && c->pxtc[l][1].usable;
}

// VX (transpose = 0) / VTX (1) of level l >= 1 on the digit engine:
// Y(a, i, b) = sum_j V_b(i, j) X(a, j, b)  or  sum_j V_b(j, i) X(a, j, b).
int tc_rot_apply(const scalit_ctx *c, int l, int transpose, const double *X, double *Y, const int *gate,
                 cudaStream_t s)
{
    const Layout &L = c->L;
    const TcLevelData &t = c->pxtc[l][transpose ? 1 : 0];
    if (!t.usable) { set_error("level %d has no tensor-core rotation plan", l + 1); return SCALIT_EUNSUP; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l];
    const i64 M = nin * blk;
    if (M > 2147483647LL || nin > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
    TcArgs g{};
    g.N = nout; g.K = nout; g.KS = t.KS; g.NT = t.NT;
    g.M = (int)M; g.Mi = nin; g.s1 = 1; g.s2 = nin * nout; g.a_sk = nin; g.c_sn = nin;
    g.A = X; g.a_sz = 0;
    g.C = Y; g.c_sz = 0;
    g.accumulate = 0;
    g.alpha = 1.0;
    g.gate = gate;
    g.err = c->tc_err;
    g.bdig = reinterpret_cast<const uint4 *>(t.dig);
    g.bexp = t.exps;
    i64 gx;
    if (blk > 1) {
        g.tpb = (int)((nin + kBM - 1) / kBM);
        g.bdig_blk = (i64)t.ntiles * t.KS * kDigits * t.NT * 2;
        g.bexp_blk = t.ntiles * t.NT;
        gx = blk * g.tpb;
    } else {
        gx = (M + kBM - 1) / kBM;
    }
    if (gx > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
    const size_t smem = 2 * (size_t)kAStepBytes + 2 * (size_t)kDigits * t.NT * 32 + (size_t)kStages * kSlab * 8 +
                        64 + 3072;
    const size_t smem_req = std::max(smem, (size_t)(116 * 1024));
    SC_CUDA(cudaFuncSetAttribute(tc_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_req));
    tc_level_kernel<<<dim3((unsigned)gx, t.ntiles, 1), kBlockTC, smem_req, s>>>(g);
    SC_CHECK_LAUNCH();
    return 0;
}

bool tc_usable(const scalit_ctx *c, int l)
{
    return c->tc[l].usable != 0;
}

int tc_level_apply(const scalit_ctx *c, int l, const double *X, double *Y, int accumulate, const double *diagV,
                   double shift, double alpha, const int *gate, cudaStream_t s, int nvec, const double *shiftv,
                   const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const TcLevelData &t = c->tc[l];
    if (!t.usable) { set_error("level %d has no tensor-core plan", l + 1); return SCALIT_EUNSUP; }
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    TcArgs g{};
    g.N = nout;
    g.K = nout;
    g.KS = t.KS;
    g.NT = t.NT;
    if (nin == 1) {
        g.M = (int)blk; g.Mi = blk; g.s1 = nout; g.s2 = 0; g.a_sk = 1; g.c_sn = 1;
        g.rowscale = nullptr;
    } else {
        const i64 M = nin * blk;
        if (M > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
        g.M = (int)M; g.Mi = nin; g.s1 = 1; g.s2 = nin * nout; g.a_sk = nin; g.c_sn = nin;
        g.rowscale = L.dep[l] ? c->DEP + L.deps[l] : nullptr;
    }
    g.A = X; g.a_sz = N;
    g.C = Y; g.c_sz = N;
    if (diagV && accumulate) { set_error("the diagonal term goes with the first level only"); return SCALIT_EINVAL; }
    g.accumulate = accumulate;
    g.alpha = alpha;
    g.diagV = diagV;
    g.diagX = X;
    g.dx_sz = N;
    g.shift = shift;
    g.shiftv = shiftv;
    g.vgate = vgate;
    g.vgate_stride = vstride;
    g.gate = gate;
    g.err = c->tc_err;
    g.bdig = reinterpret_cast<const uint4 *>(t.dig);
    g.bexp = t.exps;
    const size_t smem = 2 * (size_t)kAStepBytes + 2 * (size_t)kDigits * t.NT * 32 + (size_t)kStages * kSlab * 8 +
                        64 + 3072;
    // at least half of the SM's shared memory, so one CTA (and one TMEM owner) per SM
    const size_t smem_req = std::max(smem, (size_t)(116 * 1024));
    SC_CUDA(cudaFuncSetAttribute(tc_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_req));
    dim3 grid((g.M + kBM - 1) / kBM, t.ntiles, nvec);
    if (grid.z > 65535) { set_error("too many vectors"); return SCALIT_EINVAL; }
    tc_level_kernel<<<grid, kBlockTC, smem_req, s>>>(g);
    SC_CHECK_LAUNCH();
    return 0;
}

// Digit planes of B(k, n) = Bm[k0 + k + ldb n] for k < kc (a K chunk of a
// general K x N matrix), one thread per column n: the chunk's column exponent,
// then the digits, in the layout of cut_level_matrix.
__global__ void cut_gen_kernel(int kc, int N, int NT, int KS, const double *__restrict__ Bm, i64 ldb,
                               uint16_t *__restrict__ dig, int *__restrict__ exps)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double *col = Bm + (i64)n * ldb;
    double mx = 0.0;
    for (int k = 0; k < kc; ++k) mx = fmax(mx, fabs(col[k]));
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    exps[n] = e;
    const int tile = n / NT, nn = n % NT;
    for (int k = 0; k < kc; ++k) {
        double r = ldexp(col[k], 7 - e);
        const int ks = k / 16, kk = k % 16;
        #pragma unroll
        for (int t = 0; t < kDigits; ++t) {
            const double d = trunc(r);
            r = (r - d) * 128.0;
            const size_t base = (((size_t)tile * KS + ks) * kDigits + t) * (size_t)NT * 16;
            const size_t off = (size_t)(nn >> 3) * 128 + (size_t)(kk >> 3) * 64 + (size_t)(nn & 7) * 8 + (kk & 7);
            dig[base + off] = __bfloat16_as_ushort(__float2bfloat16_rn((float)d));   // |d| <= 127: exact
        }
    }
}

// C (M x N, column stride ldc) = A (M x K, column stride lda) B (K x N, column
// stride ldb), all FP64, on the digit engine: K in chunks of at most 256 (the
// FP32 groups' exactness bound), each chunk's product accumulated into C.
int tc_gemm_f64(const scalit_ctx *c, int M, int N, int K, const double *A, i64 lda, const double *B, i64 ldb,
                double *C, i64 ldc, cudaStream_t s)
{
    if (M <= 0 || N <= 0 || K <= 0) return 0;
    const int NT = std::min(64, (N + 15) / 16 * 16);
    const int ntiles = (N + NT - 1) / NT;
    const int kcmax = std::min(K, 256);
    const int KSmax = (kcmax + 15) / 16;
    const size_t ndig = (size_t)ntiles * KSmax * kDigits * NT * 16;
    const size_t nexp = (size_t)ntiles * NT;
    uint16_t *dig = nullptr;
    int *exps = nullptr;
    SC_CUDA(cudaMallocAsync(&dig, ndig * sizeof(uint16_t), s));
    SC_CUDA(cudaMallocAsync(&exps, nexp * sizeof(int), s));
    const size_t smem = 2 * (size_t)kAStepBytes + 2 * (size_t)kDigits * NT * 32 + (size_t)kStages * kSlab * 8 +
                        64 + 3072;
    const size_t smem_req = std::max(smem, (size_t)(116 * 1024));
    int rc = 0;
    if (cudaFuncSetAttribute(tc_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_req) !=
        cudaSuccess) { set_error("tc_gemm_f64: shared memory attribute"); rc = SCALIT_ECUDA; }
    for (int k0 = 0; k0 < K && !rc; k0 += 256) {
        const int kc = std::min(256, K - k0);
        const int KS = (kc + 15) / 16;
        if (cudaMemsetAsync(dig, 0, ndig * sizeof(uint16_t), s) != cudaSuccess ||
            cudaMemsetAsync(exps, 0, nexp * sizeof(int), s) != cudaSuccess) { rc = SCALIT_ECUDA; break; }
        cut_gen_kernel<<<(N + 127) / 128, 128, 0, s>>>(kc, N, NT, KS, B + k0, ldb, dig, exps);
        TcArgs g{};
        g.M = M; g.N = N; g.K = kc; g.KS = KS; g.NT = NT;
        g.Mi = M; g.s1 = 1; g.s2 = 0; g.a_sk = lda; g.c_sn = ldc;
        g.A = A + (i64)k0 * lda; g.a_sz = 0;
        g.C = C; g.c_sz = 0;
        g.accumulate = k0 > 0;
        g.alpha = 1.0;
        g.err = c->tc_err;
        g.bdig = reinterpret_cast<const uint4 *>(dig);
        g.bexp = exps;
        tc_level_kernel<<<dim3((M + kBM - 1) / kBM, ntiles, 1), kBlockTC, smem_req, s>>>(g);
        if (cudaGetLastError() != cudaSuccess) { set_error("tc_gemm_f64 launch"); rc = SCALIT_ECUDA; }
    }
    cudaFreeAsync(dig, s);
    cudaFreeAsync(exps, s);
    return rc;
}

int tc_check_error(scalit_ctx *c)
{
    if (!c->tc_err) return 0;
    int h = 0;
    SC_CUDA(cudaMemcpyAsync(&h, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    if (h) {
        static const char *what[] = {"", "FP64 tensor-core level product", "level-1 P*X stream",
                                     "FP32 tensor-core level product", "bounded-wait self-test",
                                     "persistent FP32 tensor-core level product",
                                     "persistent FP64 tensor-core level product"};
        set_error("%s: an mbarrier wait ran out (kernel aborted, context usable)",
                  (h >= 1 && h <= 6) ? what[h] : "device kernel");
        cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
        return SCALIT_ECUDA;
    }
    return 0;
}

// Self-test of the bounded waits: one CTA waits on an mbarrier whose expected
// transaction bytes never arrive (nothing is copied), the wait runs out after
// limit_ns, the kernel records code 4 in the context's error flag and returns
// -- the path every streaming and tensor-core kernel takes on expiry.
__global__ void wait_selftest_kernel(uint64_t limit_ns, int *err)
{
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        mbar_init(&mbar, 1);
        mbar_init_fence();
        mbar_arrive_expect_tx(&mbar, 16);      // 16 bytes that no copy delivers
        if (!mbar_wait_timed(&mbar, 0, limit_ns) && err) atomicExch(err, 4);
    }
}

int wait_selftest(scalit_ctx *c, double seconds)
{
    if (!(seconds > 0.0 && seconds <= 10.0)) { set_error("self-test wait of %g s out of (0, 10]", seconds); return SCALIT_EINVAL; }
    if (!c->tc_err) SC_CUDA(cudaMalloc(&c->tc_err, sizeof(int)));
    wait_selftest_kernel<<<1, 32, 0, c->stream>>>((uint64_t)(seconds * 1e9), c->tc_err);
    SC_CHECK_LAUNCH();
    return tc_check_error(c);
}

}  // namespace sc
