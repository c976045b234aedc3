// The OSB preconditioner P*X = V_sF..V_1 K^-1 V_1^T..V_sF^T X
// (MYPX, src/iterate/module/osb.px.h:125-219).
//
// Level 1 has one small rotation per block (VOSB level 1 holds n_1 x n_1
// matrices for every one of the myBlk(1) blocks, n_1 * N numbers in total --
// the largest array of the whole solve).  Its V_1^T, the kernel K^-1 and its
// V_1 are fused into one pass: each CTA stages the block's matrix in shared
// memory once, applies V^T, divides by the kernel, and applies V, so VOSB
// level 1 is read from HBM exactly once per application.  The outer levels
// are strided GEMMs (contract.cu).
#include "internal.cuh"
#include "ptx.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

namespace sc {

// An element of a staged matrix in the compute type (the FP32 preconditioner
// may keep its level-1 matrices in FP16).
template <class T, class TV>
__device__ __forceinline__ T vload(const TV &v)
{
    if constexpr (std::is_same<TV, __half>::value) return (T)__half2float(v);
    else return (T)v;
}

// K^-1 of the preconditioner kernel (osb.px.h:156-189).
template <class T>
__device__ __forceinline__ T kernel_div(T y, T eig, T e0, int kind, T de, T rde, T alpha_d, T beta_d)
{
    const T ade = eig - e0;
    if (kind == SCALIT_TOSBD1) {
        if (fabs(ade) <= de) return (ade < T(0)) ? -y * rde : y * rde;
        return y / ade;
    }
    if (kind == SCALIT_TOSBD2) {
        T t;
        if (fabs(ade) <= de) t = (ade < T(0)) ? (-alpha_d + beta_d * ade) : (alpha_d + beta_d * ade);
        else t = ade;
        return y / t;
    }
    return y / ade;
}

struct KernelParams {
    int kind;
    double e0, de, beta;
};

// One CTA per level-1 block.  Dynamic shared memory: n*n matrix (if it fits)
// plus two n-vectors.  nvec vectors (stride ldv) share the staged matrix; e0v
// (may be null) gives each vector its own kernel shift.
template <class T>
__global__ void __launch_bounds__(256)
px_level1_fused(int n, i64 nblk, const T *__restrict__ V, const T *__restrict__ EIG,
                const T *__restrict__ X, T *__restrict__ Y, KernelParams kp, T alpha,
                int v_in_smem, const int *gate, int nvec, i64 ldv, const double *__restrict__ e0v,
                const int *__restrict__ vgate = nullptr, int vstride = 0)
{
    if (gate && *gate) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    T *ts = xs + n;
    T *Vs = ts + n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
    const T de = T(fabs(kp.de)), rde = T(1.0 / fabs(kp.de));
    const T beta_d = T(1.0 + kp.beta), alpha_d = T(-kp.beta * fabs(kp.de));

    for (i64 b = blockIdx.x; b < nblk; b += gridDim.x) {
        const T *Vb = V + b * (i64)n * n;
        const T *Vsrc = Vb;
        __syncthreads();
        if (v_in_smem) {
            const i64 nn = (i64)n * n;
            for (i64 e = tid; e < nn; e += nt) Vs[e] = Vb[e];
            Vsrc = Vs;
        }
        for (int v = 0; v < nvec; ++v) {
            if (vgate && vgate[(i64)v * vstride]) continue;   // uniform over the CTA
            const T e0 = T(e0v ? e0v[v] : kp.e0);
            const T *xb = X + (i64)v * ldv + b * (i64)n;
            __syncthreads();
            for (int i = tid; i < n; i += nt) xs[i] = xb[i];
            __syncthreads();
            // t = V^T x: column i of V is contiguous; one warp per column.
            for (int i = warp; i < n; i += nwarp) {
                const T *col = Vsrc + (i64)i * n;
                T acc = T(0);
                for (int j = lane; j < n; j += 32) acc = fma(col[j], xs[j], acc);
                #pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0)
                    ts[i] = kernel_div<T>(acc, EIG[b * (i64)n + i], e0, kp.kind, de, rde, alpha_d, beta_d);
            }
            __syncthreads();
            // y = V t: one thread per row, consecutive rows are consecutive addresses.
            for (int i = tid; i < n; i += nt) {
                T acc = T(0);
                for (int j = 0; j < n; ++j) acc = fma(Vsrc[i + (i64)j * n], ts[j], acc);
                Y[(i64)v * ldv + b * (i64)n + i] = alpha * acc;
            }
        }
    }
}

// Streaming variant of the fused level-1 pass.  A persistent CTA walks its
// blocks while the blocks' matrices arrive as column chunks (CPW columns per
// warp, CPW * 8 * n contiguous numbers) through a ring of shared-memory slots,
// each filled by one bulk copy that completes on the slot's mbarrier.
// Column j contributes t_j = f_j (v_j . x) and then t_j v_j to y, with f_j the
// preconditioner kernel's factor for eigenvalue j, so a chunk is finished --
// both products -- as soon as it lands: each warp takes CPW columns, reduces
// their dot products together (a reduce-scatter over lane groups, then a
// broadcast of t_j) and accumulates its own rows of y in registers.  The last
// warp to finish a chunk (a shared-memory counter per slot) refills the slot
// with the chunk `ring` positions ahead, so the ring need not hold a whole
// block and HBM sees one continuous read of VOSB level 1.  The warps' partial
// y meet once per block; partials, x and the factors are double-buffered by
// block parity, so one CTA barrier per block suffices.
static constexpr int kStreamThreads = 256;
static constexpr int kStreamWarps = kStreamThreads / 32;

// The factor f with K^-1 y = f y for eigenvalue `eig` (osb.px.h:156-189).
template <class T>
__device__ __forceinline__ T kernel_factor(T eig, T e0, int kind, T de, T rde, T alpha_d, T beta_d)
{
    const T ade = eig - e0;
    if (kind == SCALIT_TOSBD1 && fabs(ade) <= de) return (ade < T(0)) ? -rde : rde;
    if (kind == SCALIT_TOSBD2 && fabs(ade) <= de)
        return T(1) / ((ade < T(0)) ? (-alpha_d + beta_d * ade) : (alpha_d + beta_d * ade));
    return T(1) / ade;
}

// Shared memory of the streaming kernel: ring mbarriers, release counters and
// last-issued chunk per slot, then the slots, then per block parity x, the
// factors and NW partial y.
__host__ __device__ constexpr size_t px1_stream_head(int ring)
{
    return (((size_t)ring * 16 + 127) & ~(size_t)127);
}

// FULL: n == 32 * RPL, every lane holds RPL rows and no row test is needed.
// CPW (2 or 4): columns per warp and chunk.  TV: the matrices' storage type
// (T, or FP16 for the FP32 preconditioner: half the bytes streamed).
template <class T, class TV, int RPL, bool FULL, int CPW>
__global__ void __launch_bounds__(kStreamThreads, sizeof(T) == 4 ? 4 : 2)
px_level1_stream(int n, i64 nblk, const TV *__restrict__ V, const T *__restrict__ EIG,
                 const T *__restrict__ X, T *__restrict__ Y, KernelParams kp, T alpha, int nc, int ring,
                 const int *gate, int *err)
{
    if (gate && *gate) return;
    extern __shared__ __align__(16) unsigned char smem_stream[];
    __shared__ int abort_flag;
    constexpr int NW = kStreamWarps, kChunkCols = CPW * kStreamWarps;
    static_assert(CPW == 2 || CPW == 4, "two or four columns per warp");
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_stream);
    int *relcnt = reinterpret_cast<int *>(full + ring);         // warps done with the slot's chunks
    int *last = relcnt + ring;                                  // the chunk last issued into the slot
    const int slot_elems = kChunkCols * n;
    TV *slots = reinterpret_cast<TV *>(smem_stream + px1_stream_head(ring));
    T *vec0 = reinterpret_cast<T *>(slots + ring * slot_elems); // per parity: x, f, NW partials
    const int vstride = (2 + NW) * n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const T e0 = T(kp.e0), de = T(fabs(kp.de)), rde = T(1.0 / fabs(kp.de));
    const T beta_d = T(1.0 + kp.beta), alpha_d = T(-kp.beta * fabs(kp.de));

    // chunk and slot counters are plain ints advanced step by step: the loops
    // hold no 64-bit division or remainder
    const int kblocks = (int)((nblk - blockIdx.x + gridDim.x - 1) / gridDim.x);   // blocks of this CTA
    const int G = kblocks * nc;                                                  // its chunks
    auto issue = [&](int g, int slot) {
        const int kk = g / nc, c0 = (g - kk * nc) * kChunkCols;
        const i64 b = blockIdx.x + (i64)kk * gridDim.x;
        const int cols = min(kChunkCols, n - c0);
        const uint32_t bytes = (uint32_t)(sizeof(TV) * (size_t)cols * n);
        last[slot] = g;
        mbar_arrive_expect_tx(&full[slot], bytes);
        bulk_g2s(slots + slot * slot_elems, V + b * (i64)n * n + (i64)c0 * n, bytes, &full[slot]);
    };
    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < ring; ++i) {
            mbar_init(&full[i], 1);
            relcnt[i] = 0;
            last[i] = -1;
        }
        mbar_init_fence();
        for (int g = 0; g < G && g < ring; ++g) issue(g, g);
    }
    // x and the factors of the first block; each later block's are written
    // into the other parity before the previous block's barrier
    if (kblocks > 0 && tid < n) {
        vec0[tid] = X[(i64)blockIdx.x * n + tid];
        vec0[n + tid] = kernel_factor<T>(EIG[(i64)blockIdx.x * n + tid], e0, kp.kind, de, rde, alpha_d, beta_d);
    }
    __syncthreads();
    int slot = 0;                                       // the current chunk's slot and phase
    uint32_t par = 0;
    int k = 0;
    for (; k < kblocks; ++k) {
        const i64 b = blockIdx.x + (i64)k * gridDim.x;
        T *xs = vec0 + (k & 1) * vstride, *fs = xs + n, *part = fs + n;
        const bool more = k + 1 < kblocks && tid < n;
        T xn = T(0), en = T(0);
        if (more) {
            const i64 bn = b + gridDim.x;
            xn = X[bn * n + tid];
            en = EIG[bn * n + tid];
        }
        T xr[RPL], acc[RPL];
        #pragma unroll
        for (int r = 0; r < RPL; ++r) {
            const int row = lane + 32 * r;
            xr[r] = (FULL || row < n) ? xs[row] : T(0);
            acc[r] = T(0);
        }
        for (int c = 0; c < nc; ++c) {
            const int g = k * nc + c;
            if (!__all_sync(0xffffffffu, mbar_wait_timed(&full[slot], par))) { abort_flag = 1; break; }
            const TV *chunk = slots + slot * slot_elems + lane;
            const int c0 = c * kChunkCols, cols = min(kChunkCols, n - c0);
            // the warp's CPW columns, each element read once from shared
            // memory (columns past the block's last are zero: warp-uniform)
            T v[CPW][RPL], d[CPW];
            #pragma unroll
            for (int q = 0; q < CPW; ++q) {
                const int j = warp + q * NW;
                const TV *col = chunk + j * n;
                d[q] = T(0);
                #pragma unroll
                for (int r = 0; r < RPL; ++r) {
                    v[q][r] = (j < cols && (FULL || lane + 32 * r < n)) ? vload<T>(col[32 * r]) : T(0);
                    d[q] = fma(v[q][r], xr[r], d[q]);
                }
            }
            // reduce-scatter: at each of the first log2(CPW) shuffle levels
            // the two lane groups swap the columns they do not keep, so lane
            // group q = lane / (32 / CPW) ends with column q's full sum after
            // five levels; t_q is then broadcast from the group's first lane
            T keep;
            if constexpr (CPW == 2) {
                const bool h = lane & 16;
                keep = (h ? d[1] : d[0]) + __shfl_xor_sync(0xffffffffu, h ? d[0] : d[1], 16);
            } else {
                const bool h1 = lane & 16, h2 = lane & 8;
                const T k0 = (h1 ? d[2] : d[0]) + __shfl_xor_sync(0xffffffffu, h1 ? d[0] : d[2], 16);
                const T k1 = (h1 ? d[3] : d[1]) + __shfl_xor_sync(0xffffffffu, h1 ? d[1] : d[3], 16);
                keep = (h2 ? k1 : k0) + __shfl_xor_sync(0xffffffffu, h2 ? k0 : k1, 8);
            }
            #pragma unroll
            for (int o = 32 / CPW / 2; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
            const int qh = lane / (32 / CPW), jh = warp + qh * NW;
            const T th = jh < cols ? keep * fs[c0 + jh] : T(0);
            #pragma unroll
            for (int q = 0; q < CPW; ++q) {
                const T tq = __shfl_sync(0xffffffffu, th, q * (32 / CPW));
                #pragma unroll
                for (int r = 0; r < RPL; ++r) acc[r] = fma(v[q][r], tq, acc[r]);
            }
            // release; the last warp out refills the slot
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                if ((atomicAdd(&relcnt[slot], 1) + 1) % NW == 0) {      // counts NW per use of the slot
                    __threadfence_block();
                    if (g + ring < G) {
                        fence_proxy_async_smem();
                        issue(g + ring, slot);
                    }
                }
            }
            if (++slot == ring) { slot = 0; par ^= 1u; }
        }
        #pragma unroll
        for (int r = 0; r < RPL; ++r) {
            const int row = lane + 32 * r;
            if (FULL || row < n) part[warp * n + row] = acc[r];
        }
        if (more) {
            T *xo = vec0 + ((k + 1) & 1) * vstride;
            xo[tid] = xn;
            xo[n + tid] = kernel_factor<T>(en, e0, kp.kind, de, rde, alpha_d, beta_d);
        }
        __syncthreads();
        if (abort_flag) break;
        for (int i = tid; i < n; i += kStreamThreads) {
            T y = T(0);
            #pragma unroll
            for (int w = 0; w < NW; ++w) y += part[w * n + i];
            Y[b * (i64)n + i] = alpha * y;
        }
    }
    if (abort_flag && tid == 0) {
        if (err) atomicExch(err, 2);
        // every warp has stopped: let the latest copy into each slot land
        // before the CTA's shared memory is released
        for (int s = 0; s < ring; ++s)
            if (last[s] >= 0) mbar_wait_timed(&full[s], (uint32_t)((last[s] / ring) & 1));
    }
}

// Batched y_b = V_b x_b (transpose = 0) or V_b^T x_b (transpose = 1), one CTA per block.
template <class T>
__global__ void __launch_bounds__(256)
bgemv_kernel(int n, i64 nblk, const T *__restrict__ V, const T *__restrict__ X, T *__restrict__ Y,
             int transpose, const int *gate)
{
    if (gate && *gate) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
    for (i64 b = blockIdx.x; b < nblk; b += gridDim.x) {
        const T *Vb = V + b * (i64)n * n;
        __syncthreads();
        for (int i = tid; i < n; i += nt) xs[i] = X[b * (i64)n + i];
        __syncthreads();
        if (transpose) {
            for (int i = warp; i < n; i += nwarp) {
                const T *col = Vb + (i64)i * n;
                T acc = T(0);
                for (int j = lane; j < n; j += 32) acc = fma(col[j], xs[j], acc);
                #pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) Y[b * (i64)n + i] = acc;
            }
        } else {
            for (int i = tid; i < n; i += nt) {
                T acc = T(0);
                for (int j = 0; j < n; ++j) acc = fma(Vb[i + (i64)j * n], xs[j], acc);
                Y[b * (i64)n + i] = acc;
            }
        }
    }
}

static int grid_for(i64 nblk)
{
    const i64 cap = 152LL * 64;
    return (int)(nblk < cap ? nblk : cap);
}

template <class T>
int bgemv(int nout, int blk, const T *V, const T *X, T *Y, int transpose, const int *gate,
          cudaStream_t s)
{
    if (blk <= 0 || nout <= 0) return 0;
    const size_t sm = sizeof(T) * (size_t)nout;
    bgemv_kernel<T><<<grid_for(blk), 256, sm, s>>>(nout, blk, V, X, Y, transpose, gate);
    SC_CHECK_LAUNCH();
    return 0;
}

template int bgemv<double>(int, int, const double *, const double *, double *, int, const int *, cudaStream_t);
template int bgemv<float>(int, int, const float *, const float *, float *, int, const int *, cudaStream_t);

static constexpr size_t kMaxDynSmem = 220 * 1024;

// Shared memory of one SM and what each resident CTA loses to the runtime.
static constexpr size_t kSmSmem = 228 * 1024;
static constexpr size_t kCtaReserve = 1024 + 128;   // runtime reserve + static shared data

// CTAs per SM for the streaming kernel: an explicit choice from the
// environment (SCALIT_PX1_CTAS, a tuning override), else the most CTAs that
// are resident at once (registers and shared memory) with a ring of at least
// two chunks -- measured on GB300, more warps per SM beat a deeper ring.
// Returns 0 when no count fits, else the count, with the deepest ring (up to
// four blocks) that it leaves room for.
static int px1_stream_shape(const void *fn, size_t chunk, int nc, size_t vecs, int &ring)
{
    static const int forced = [] {
        const char *e = getenv("SCALIT_PX1_CTAS");
        return e ? atoi(e) : 0;
    }();
    int best = 0, best_ring = 0;
    for (int per_sm = 1; per_sm <= 8; ++per_sm) {
        const size_t budget = std::min(kMaxDynSmem, kSmSmem / per_sm - kCtaReserve);
        if (budget <= vecs + 128 + 2 * (chunk + 16)) break;
        const int r = (int)std::min<size_t>((budget - vecs - 128) / (chunk + 16), (size_t)4 * nc);
        int resident = 0;
        const size_t smem = px1_stream_head(r) + (size_t)r * chunk + vecs;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fn, kStreamThreads, smem) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        if (resident < per_sm) break;
        best = per_sm;
        best_ring = r;
        if (per_sm == forced) break;
    }
    ring = best_ring;
    return best;
}

// Launch of the streaming kernel; returns 1 when it does not apply (no ring
// of two chunks fits), so the caller takes the one-CTA-per-block kernel.
template <class T, class TV, int RPL, bool FULL, int CPW>
static int launch_px1_stream_as(int n, i64 nblk, const TV *V, const T *EIG, const T *X, T *Y, KernelParams kp,
                                T alpha, const int *gate, int *err, cudaStream_t s)
{
    static int configured = -1;
    static int shape_n[257], shape_cta[257], shape_ring[257];   // per block size, filled on first use
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaFuncSetAttribute(px_level1_stream<T, TV, RPL, FULL, CPW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem));
        for (int i = 0; i <= 256; ++i) shape_n[i] = 0;
        configured = dev;
    }
    constexpr int kChunkCols = CPW * kStreamWarps;
    const size_t chunk = sizeof(TV) * (size_t)kChunkCols * n;
    const int nc = (n + kChunkCols - 1) / kChunkCols;
    const size_t vecs = sizeof(T) * (size_t)n * 2 * (2 + kStreamWarps);
    if (!shape_n[n]) {
        int ring = 0;
        shape_cta[n] = px1_stream_shape(reinterpret_cast<const void *>(px_level1_stream<T, TV, RPL, FULL, CPW>),
                                        chunk, nc, vecs, ring);
        shape_ring[n] = ring;
        shape_n[n] = 1;
    }
    const int per_sm = shape_cta[n], ring = shape_ring[n];
    if (per_sm == 0) return 1;
    if ((nblk / (152 * per_sm) + 1) * nc > 2147483647LL) return 1;   // a CTA counts its chunks in an int
    const size_t smem = px1_stream_head(ring) + (size_t)ring * chunk + vecs;
    const int grid = (int)std::min<i64>(nblk, 152 * per_sm);
    px_level1_stream<T, TV, RPL, FULL, CPW><<<grid, kStreamThreads, smem, s>>>(n, nblk, V, EIG, X, Y, kp, alpha,
                                                                               nc, ring, gate, err);
    SC_CHECK_LAUNCH();
    return 0;
}

template <class T, class TV, int RPL>
static int launch_px1_stream(int n, i64 nblk, const TV *V, const T *EIG, const T *X, T *Y, KernelParams kp,
                             T alpha, const int *gate, int *err, cudaStream_t s)
{
    // four columns per warp halve the per-chunk overhead; two keep the
    // register footprint of long columns in bounds
    constexpr int CPW = RPL <= 5 ? 4 : 2;
    if (n == 32 * RPL)
        return launch_px1_stream_as<T, TV, RPL, true, CPW>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    return launch_px1_stream_as<T, TV, RPL, false, CPW>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
}

// The streaming kernel with matrices stored as TV; returns 1 when it does
// not apply (chunks and bases must be 16-byte aligned).
template <class T, class TV>
static int launch_px1_streamed(int n, i64 nblk, const TV *V, const T *EIG, const T *X, T *Y,
                               KernelParams kp, T alpha, const int *gate, int *err, cudaStream_t s)
{
    const bool aligned = ((reinterpret_cast<uintptr_t>(V) & 15) == 0) && ((sizeof(TV) * (size_t)n * n) % 16 == 0) &&
                         ((sizeof(TV) * (size_t)n) % 16 == 0 || sizeof(TV) == sizeof(T));
    if (!(n >= 1 && n <= 256 && nblk >= 1 && aligned)) return 1;
    switch ((n + 31) / 32) {
    case 1: return launch_px1_stream<T, TV, 1>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 2: return launch_px1_stream<T, TV, 2>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 3: return launch_px1_stream<T, TV, 3>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 4: return launch_px1_stream<T, TV, 4>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 5: return launch_px1_stream<T, TV, 5>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 6: return launch_px1_stream<T, TV, 6>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    case 7: return launch_px1_stream<T, TV, 7>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    default: return launch_px1_stream<T, TV, 8>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
    }
}

template <class T>
static int launch_px1(int n, i64 nblk, const T *V, const T *EIG, const T *X, T *Y,
                      KernelParams kp, T alpha, const int *gate, int *err, cudaStream_t s)
{
    // the streaming kernel: chunks and bases 16-byte aligned
    {
        const int rc = launch_px1_streamed<T, T>(n, nblk, V, EIG, X, Y, kp, alpha, gate, err, s);
        if (rc <= 0) return rc;
    }
    const size_t vec = sizeof(T) * 2 * (size_t)n;
    const size_t mat = sizeof(T) * (size_t)n * n;
    const int v_in_smem = (vec + mat <= kMaxDynSmem) ? 1 : 0;
    const size_t sm = vec + (v_in_smem ? mat : 0);
    static int configured = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaFuncSetAttribute(px_level1_fused<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kMaxDynSmem));
        configured = dev;
    }
    px_level1_fused<T><<<grid_for(nblk), 256, sm, s>>>(n, nblk, V, EIG, X, Y, kp, alpha, v_in_smem, gate, 1, 0,
                                                       nullptr);
    SC_CHECK_LAUNCH();
    return 0;
}

template <class T> static const T *pickp(const double *d, const float *f);
template <> const double *pickp<double>(const double *d, const float *) { return d; }
template <> const float *pickp<float>(const double *, const float *f) { return f; }

// VX / VTX of level l >= 2: FP64 on the tensor-core digit engine when it is
// the context's FP64 engine, otherwise the strided GEMM.
template <class T>
static int rotate(const scalit_ctx *c, int l, int transpose, const T *V, const T *in, T *out, const int *gate,
                  cudaStream_t s)
{
    const Layout &L = c->L;
    if constexpr (std::is_same<T, double>::value) {
        if (tc_px_usable(c, l)) return tc_rot_apply(c, l, transpose, in, out, gate, s);
    } else {
        if (tc32_px_usable(c, l)) return tc32_rot_apply(c, l, transpose, in, out, gate, s, 1);
    }
    return level_rotate<T>((int)L.dim[l], L.n[l], (int)L.blk[l], V + L.vs[l], in, out, transpose, gate, s);
}

// VX (transpose = 0) or VTX (transpose = 1) of one level, FP64, out of place:
// the engines of the real P*X (level 1 by the batched block GEMV).
int px_rotate(const scalit_ctx *c, int l, int transpose, const double *in, double *out, const int *gate,
              cudaStream_t s)
{
    const Layout &L = c->L;
    if (l == 0) return level_rotate<double>(1, L.n[0], (int)L.blk[0], c->VOSB + L.vs[0], in, out, transpose, gate, s);
    return rotate<double>(c, l, transpose, c->VOSB, in, out, gate, s);
}

// MYPX with the TOSBW kernel (osb.px.h:191-206): the level-1 rotations are
// not fused with the kernel step, whose window entries couple blocks.
// Stages: V^T of levels sF..1, the window step in place, V of levels 1..sF.
template <class T>
static int px_vec_window(const scalit_ctx *c, int npc, const T *X, T *Y, T *tmp, T alpha, const int *gate,
                         cudaStream_t s)
{
    const Layout &L = c->L;
    if (!(c->osbw_len > 0 && c->osbw_valid)) {
        set_error("TOSBW P*X without a window for the current preconditioner: call scalit_build_osbw again");
        return SCALIT_ESTATE;
    }
    const T *V = pickp<T>(c->VOSB, c->VOSBf);
    const T *EIG = pickp<T>(c->EIG0, c->EIG0f);
    const int S = 2 * L.nlev;
    T *buf[2] = {Y, tmp};
    const T *in = X;
    int stage = 0, rc;
    for (int l = L.nlev - 1; l >= 0; --l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = (l == 0) ? level_rotate<T>(1, L.n[0], (int)L.blk[0], V + L.vs[0], in, out, 1, gate, s)
                      : rotate<T>(c, l, 1, V, in, out, gate, s);
        if (rc) return rc;
        in = out;
    }
    rc = osbw_window_apply<T>(c, const_cast<T *>(in), EIG, npc == SCALIT_TA0 ? 0.0 : c->E0, alpha, gate, s);
    if (rc) return rc;
    for (int l = 0; l < L.nlev; ++l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = (l == 0) ? level_rotate<T>(1, L.n[0], (int)L.blk[0], V + L.vs[0], in, out, 0, gate, s)
                      : rotate<T>(c, l, 0, V, in, out, gate, s);
        if (rc) return rc;
        in = out;
    }
    return 0;
}

template <class T>
int px_vec(const scalit_ctx *c, int npc, const T *X, T *Y, T *tmp, T alpha, const int *gate,
           cudaStream_t s)
{
    const Layout &L = c->L;
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
    if (c->osb_kind == SCALIT_TOSBW) return px_vec_window<T>(c, npc, X, Y, tmp, alpha, gate, s);
    const T *V = pickp<T>(c->VOSB, c->VOSBf);
    const T *EIG = pickp<T>(c->EIG0, c->EIG0f);
    KernelParams kp{c->osb_kind, npc == SCALIT_TA0 ? 0.0 : c->E0, c->osb_de, c->osb_beta};
    // Stages: V^T of levels sF..2, fused level 1, V of levels 2..sF.
    const int S = 2 * L.nlev - 1;
    T *buf[2] = {Y, tmp};
    const T *in = X;
    int stage = 0, rc;
    for (int l = L.nlev - 1; l >= 1; --l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = rotate<T>(c, l, 1, V, in, out, gate, s);
        if (rc) return rc;
        in = out;
    }
    ++stage;
    {
        T *out = buf[(S - stage) % 2];
        rc = 1;
        if constexpr (std::is_same<T, float>::value) {
            // level-1 matrices in FP16 (scalit_set_fp32_px_storage): half the bytes
            if (c->VOSBh)
                rc = launch_px1_streamed<float, __half>(L.n[0], L.blk[0], static_cast<const __half *>(c->VOSBh), EIG,
                                                        in, out, kp, alpha, gate, c->tc_err, s);
        }
        if (rc > 0) rc = launch_px1<T>(L.n[0], L.blk[0], V + L.vs[0], EIG, in, out, kp, alpha, gate, c->tc_err, s);
        if (rc) return rc;
        in = out;
    }
    for (int l = 1; l < L.nlev; ++l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = rotate<T>(c, l, 0, V, in, out, gate, s);
        if (rc) return rc;
        in = out;
    }
    return 0;
}

template int px_vec<double>(const scalit_ctx *, int, const double *, double *, double *, double, const int *, cudaStream_t);

__global__ void f64_to_f16_kernel(i64 n, const double *__restrict__ x, __half *__restrict__ y)
{
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        y[i] = __double2half(x[i]);
}

// The FP16 copy of the level-1 matrices for the FP32 P*X, made from the FP64
// preconditioner when the context asks for it (after every build or load),
// freed otherwise.
int px_half_prepare(scalit_ctx *c)
{
    const Layout &L = c->L;
    const bool want = c->px_bits == 16 && c->osb_built && L.n[0] % 8 == 0;
    if (!want) {
        if (c->VOSBh) { cudaFree(c->VOSBh); c->VOSBh = nullptr; }
        return 0;
    }
    const i64 n = L.blk[0] * (i64)L.n[0] * L.n[0];
    if (!c->VOSBh) SC_CUDA(cudaMalloc(&c->VOSBh, sizeof(__half) * (size_t)n));
    const int grid = (int)std::min<i64>((n + 255) / 256, 152 * 16);
    f64_to_f16_kernel<<<grid, 256, 0, c->stream>>>(n, c->VOSB + L.vs[0], static_cast<__half *>(c->VOSBh));
    SC_CHECK_LAUNCH();
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}
// P*X of nvec vectors (stride N) at once, vector v with its own kernel shift
// e0v[v] (device): the level-1 matrices are staged once per block for all the
// vectors, and the outer rotations fold the vectors into the GEMM rows.
template <class T>
int px_multi(const scalit_ctx *c, const T *X, T *Y, T *tmp, int nvec, const double *e0v, const int *gate,
             cudaStream_t s, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
    if (c->osb_kind == SCALIT_TOSBW) {
        set_error("the OSBW window is factored for one shift: per-vector shifts need TOSB, TOSBD1 or TOSBD2");
        return SCALIT_EUNSUP;
    }
    if (nvec < 1) return 0;
    const T *V = pickp<T>(c->VOSB, c->VOSBf);
    const T *EIG = pickp<T>(c->EIG0, c->EIG0f);
    KernelParams kp{c->osb_kind, c->E0, c->osb_de, c->osb_beta};
    const i64 N = L.N;
    const int S = 2 * L.nlev - 1;
    T *buf[2] = {Y, tmp};
    const T *in = X;
    int stage = 0, rc;
    auto rot = [&](int l, int transpose, const T *a, T *o) -> int {
        const i64 nin = L.dim[l];
        const int nout = L.n[l];
        if constexpr (std::is_same<T, double>::value) {
            if (tc_px_usable(c, l)) {
                for (int v = 0; v < nvec; ++v) {
                    int r = tc_rot_apply(c, l, transpose, a + (i64)v * N, o + (i64)v * N, gate, s);
                    if (r) return r;
                }
                return 0;
            }
        } else {
            if (tc32_px_usable(c, l)) return tc32_rot_apply(c, l, transpose, a, o, gate, s, nvec, vgate, vstride);
        }
        // batch z = v blk + b: vector v's block b sits at z nin nout (N = nin nout blk)
        const i64 nb = L.blk[l] * nvec;
        if (nb > 65535) { set_error("level %d: %lld blocks x vectors too many", l + 1, (long long)nb); return SCALIT_EINVAL; }
        GemmArgs<T> g{};
        g.K = nout; g.accumulate = 0; g.alpha = T(1); g.gate = gate;
        g.rowscale = nullptr; g.diagV = nullptr;
        g.M = (int)nin; g.N = nout; g.batch = (int)nb;
        g.Mi = nin; g.s1 = 1; g.s2 = 0;
        g.A = a; g.a_sk = nin; g.a_sz = nin * nout;
        g.B = V + L.vs[l]; g.b_sz = (i64)nout * nout; g.b_mod = (int)L.blk[l];
        g.vgate = vgate; g.vgate_stride = vstride; g.vgate_div = (int)L.blk[l];
        if (!transpose) { g.b_sk = nout; g.b_sn = 1; }
        else { g.b_sk = 1; g.b_sn = nout; }
        g.C = o; g.c_sn = nin; g.c_sz = nin * nout;
        return launch_gemm<T>(g, s);
    };
    for (int l = L.nlev - 1; l >= 1; --l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = rot(l, 1, in, out);
        if (rc) return rc;
        in = out;
    }
    ++stage;
    {
        T *out = buf[(S - stage) % 2];
        const int n = L.n[0];
        const size_t vec = sizeof(T) * 2 * (size_t)n;
        const size_t mat = sizeof(T) * (size_t)n * n;
        const int v_in_smem = (vec + mat <= kMaxDynSmem) ? 1 : 0;
        const size_t sm = vec + (v_in_smem ? mat : 0);
        static int configured = -1;
        int dev = 0;
        cudaGetDevice(&dev);
        if (configured != dev) {
            SC_CUDA(cudaFuncSetAttribute(px_level1_fused<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxDynSmem));
            configured = dev;
        }
        px_level1_fused<T><<<grid_for(L.blk[0]), 256, sm, s>>>(n, L.blk[0], V + L.vs[0], EIG, in, out, kp, T(1),
                                                               v_in_smem, gate, nvec, N, e0v, vgate, vstride);
        SC_CHECK_LAUNCH();
        in = out;
    }
    for (int l = 1; l < L.nlev; ++l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = rot(l, 0, in, out);
        if (rc) return rc;
        in = out;
    }
    return 0;
}

template int px_multi<double>(const scalit_ctx *, const double *, double *, double *, int, const double *, const int *, cudaStream_t, const int *, int);
template int px_multi<float>(const scalit_ctx *, const float *, float *, float *, int, const double *, const int *, cudaStream_t, const int *, int);

template int px_vec<float>(const scalit_ctx *, int, const float *, float *, float *, float, const int *, cudaStream_t);

}  // namespace sc
