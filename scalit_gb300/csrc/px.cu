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

#include <algorithm>
#include <type_traits>

namespace sc {

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

// Streaming variant of the fused level-1 pass: a persistent CTA walks its
// blocks while the blocks' matrices arrive as column chunks (kChunkCols
// columns = kChunkCols * n contiguous numbers) through a ring of shared-memory
// slots, each filled by one bulk copy that completes on the slot's mbarrier.
// Phase 1 (t = V^T x, then K^-1) takes a chunk as soon as it lands; phase 2
// (y = V t, one warp per column, every lane accumulating its own rows) frees
// each slot once all warps are past it, and the slot is refilled right away
// with the chunk `ring` positions ahead -- the next block's columns stream in
// while this block finishes, so HBM sees one continuous read of VOSB level 1.
static constexpr int kChunkCols = 16;
static constexpr int kStreamThreads = 256;

template <class T, int RPL>
__global__ void __launch_bounds__(kStreamThreads)
px_level1_stream(int n, i64 nblk, const T *__restrict__ V, const T *__restrict__ EIG,
                 const T *__restrict__ X, T *__restrict__ Y, KernelParams kp, T alpha, int nc, int ring,
                 const int *gate, int *err)
{
    if (gate && *gate) return;
    extern __shared__ __align__(16) unsigned char smem_stream[];
    __shared__ int abort_flag;
    constexpr int NW = kStreamThreads / 32;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem_stream);
    const size_t slot_elems = (size_t)kChunkCols * n;
    T *slots = reinterpret_cast<T *>(smem_stream + (((size_t)ring * 8 + 127) & ~(size_t)127));
    T *xs = slots + (size_t)ring * slot_elems;
    T *ts = xs + n;
    T *es = ts + n;                                     // the block's EIG0
    T *part = es + n;                                   // NW x n
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const T e0 = T(kp.e0), de = T(fabs(kp.de)), rde = T(1.0 / fabs(kp.de));
    const T beta_d = T(1.0 + kp.beta), alpha_d = T(-kp.beta * fabs(kp.de));

    const i64 kblocks = (nblk - blockIdx.x + gridDim.x - 1) / gridDim.x;   // blocks of this CTA
    const i64 G = kblocks * nc;                                            // its chunks
    auto issue = [&](i64 g) {
        const i64 b = blockIdx.x + (g / nc) * (i64)gridDim.x;
        const int c0 = (int)(g % nc) * kChunkCols;
        const int cols = min(kChunkCols, n - c0);
        const uint32_t bytes = (uint32_t)(sizeof(T) * (size_t)cols * n);
        const int slot = (int)(g % ring);
        mbar_arrive_expect_tx(&mbar[slot], bytes);
        bulk_g2s(slots + (size_t)slot * slot_elems, V + b * (i64)n * n + (i64)c0 * n, bytes, &mbar[slot]);
    };
    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < ring; ++i) mbar_init(&mbar[i], 1);
        mbar_init_fence();
        for (i64 g = 0; g < G && g < ring; ++g) issue(g);
    }
    // X and EIG0 of the first block; later blocks' are fetched during the
    // previous block's phase 2 (one value per thread, n <= 256)
    if (kblocks > 0 && tid < n) {
        xs[tid] = X[(i64)blockIdx.x * n + tid];
        es[tid] = EIG[(i64)blockIdx.x * n + tid];
    }
    __syncthreads();
    i64 issued = G < ring ? G : ring;    // meaningful in thread 0
    i64 k = 0;
    for (; k < kblocks; ++k) {
        const i64 b = blockIdx.x + k * (i64)gridDim.x;
        // phase 1: t = K^-1 V^T x.  One warp per column, lanes over rows; two
        // shuffle levels leave 8 partial dots per column in part[], summed and
        // divided by the kernel below with one thread per column.
        for (int c = 0; c < nc; ++c) {
            const i64 g = k * nc + c;
            if (!mbar_wait(&mbar[g % ring], (uint32_t)((g / ring) & 1))) { abort_flag = 1; break; }
            const T *chunk = slots + (size_t)(g % ring) * slot_elems;
            const int c0 = c * kChunkCols, cols = min(kChunkCols, n - c0);
            for (int j = warp; j < cols; j += NW) {
                const T *col = chunk + (size_t)j * n;
                T acc = T(0);
                #pragma unroll
                for (int r = 0; r < RPL; ++r) {
                    const int row = lane + 32 * r;
                    if (row < n) acc = fma(col[row], xs[row], acc);
                }
                acc += __shfl_xor_sync(0xffffffffu, acc, 16);
                acc += __shfl_xor_sync(0xffffffffu, acc, 8);
                if (lane < 8) part[(c0 + j) * 8 + lane] = acc;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        for (int i = tid; i < n; i += kStreamThreads) {
            const T *pp = part + i * 8;
            const T d = ((pp[0] + pp[1]) + (pp[2] + pp[3])) + ((pp[4] + pp[5]) + (pp[6] + pp[7]));
            ts[i] = kernel_div<T>(d, es[i], e0, kp.kind, de, rde, alpha_d, beta_d);
        }
        __syncthreads();
        // phase 2: y = V t, releasing the slots in order; meanwhile the next
        // block's X and EIG0 are on their way into registers
        const bool more = k + 1 < kblocks && tid < n;
        T xn = T(0), en = T(0);
        if (more) {
            const i64 bn = b + gridDim.x;
            xn = X[bn * n + tid];
            en = EIG[bn * n + tid];
        }
        T acc[RPL];
        #pragma unroll
        for (int r = 0; r < RPL; ++r) acc[r] = T(0);
        for (int c = 0; c < nc; ++c) {
            const i64 g = k * nc + c;
            const T *chunk = slots + (size_t)(g % ring) * slot_elems;
            const int c0 = c * kChunkCols, cols = min(kChunkCols, n - c0);
            for (int j = warp; j < cols; j += NW) {
                const T *col = chunk + (size_t)j * n;
                const T tj = ts[c0 + j];
                #pragma unroll
                for (int r = 0; r < RPL; ++r) {
                    const int row = lane + 32 * r;
                    if (row < n) acc[r] = fma(col[row], tj, acc[r]);
                }
            }
            __syncthreads();
            if (tid == 0 && g + ring < G) {
                fence_proxy_async_smem();
                issue(g + ring);
                issued = g + ring + 1;
            }
        }
        #pragma unroll
        for (int r = 0; r < RPL; ++r) {
            const int row = lane + 32 * r;
            if (row < n) part[warp * n + row] = acc[r];
        }
        __syncthreads();
        for (int i = tid; i < n; i += kStreamThreads) {
            T y = T(0);
            #pragma unroll
            for (int w = 0; w < NW; ++w) y += part[w * n + i];
            Y[b * (i64)n + i] = alpha * y;
        }
        if (more) { xs[tid] = xn; es[tid] = en; }
        __syncthreads();
    }
    if (abort_flag && tid == 0) {
        if (err) atomicExch(err, 2);
        // let every copy this CTA issued land before the CTA's shared memory is released
        for (i64 g = k * nc; g < issued; ++g) mbar_wait(&mbar[g % ring], (uint32_t)((g / ring) & 1));
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

template <class T, int RPL>
static int launch_px1_stream(int n, i64 nblk, const T *V, const T *EIG, const T *X, T *Y, KernelParams kp,
                             T alpha, int nc, int ring, size_t smem, int per_sm, const int *gate, int *err,
                             cudaStream_t s)
{
    static int configured = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (configured != dev) {
        SC_CUDA(cudaFuncSetAttribute(px_level1_stream<T, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kMaxDynSmem));
        configured = dev;
    }
    const int grid = (int)std::min<i64>(nblk, 152 * per_sm);
    px_level1_stream<T, RPL><<<grid, kStreamThreads, smem, s>>>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring,
                                                                gate, err);
    SC_CHECK_LAUNCH();
    return 0;
}

template <class T>
static int launch_px1(int n, i64 nblk, const T *V, const T *EIG, const T *X, T *Y,
                      KernelParams kp, T alpha, const int *gate, int *err, cudaStream_t s)
{
    // the streaming kernel: whole blocks fit the ring, chunks and bases 16-byte aligned
    const size_t chunk = sizeof(T) * (size_t)kChunkCols * n;
    const int nc = (n + kChunkCols - 1) / kChunkCols;
    const size_t fixed = sizeof(T) * (size_t)n * (3 + kStreamThreads / 32) + 256 + 64 * 8;
    // two CTAs per SM when a ring of one block fits in half the shared memory
    // (one CTA's barriers then overlap the other's copies), else one CTA with
    // the deepest ring that fits
    const size_t half = 113 * 1024;
    const int ring2 = (half > fixed) ? (int)std::min<size_t>((half - fixed) / chunk, (size_t)nc) : 0;
    const int per_sm = (ring2 >= nc) ? 2 : 1;
    const int ring = (per_sm == 2) ? ring2 : (int)std::min<size_t>((kMaxDynSmem - fixed) / chunk, (size_t)3 * nc);
    const bool aligned = ((reinterpret_cast<uintptr_t>(V) & 15) == 0) && ((sizeof(T) * (size_t)n * n) % 16 == 0);
    if (n <= 256 && ring >= nc && nblk >= 1 && aligned) {
        const size_t smem = (((size_t)ring * 8 + 127) & ~(size_t)127) + (size_t)ring * chunk +
                            sizeof(T) * (size_t)n * (3 + kStreamThreads / 32);
        switch ((n + 31) / 32) {
        case 1: return launch_px1_stream<T, 1>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 2: return launch_px1_stream<T, 2>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 3: return launch_px1_stream<T, 3>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 4: return launch_px1_stream<T, 4>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 5: return launch_px1_stream<T, 5>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 6: return launch_px1_stream<T, 6>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        case 7: return launch_px1_stream<T, 7>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        default: return launch_px1_stream<T, 8>(n, nblk, V, EIG, X, Y, kp, alpha, nc, ring, smem, per_sm, gate, err, s);
        }
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

template <class T>
int px_vec(const scalit_ctx *c, int npc, const T *X, T *Y, T *tmp, T alpha, const int *gate,
           cudaStream_t s)
{
    const Layout &L = c->L;
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
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
        rc = launch_px1<T>(L.n[0], L.blk[0], V + L.vs[0], EIG, in, out, kp, alpha, gate, c->tc_err, s);
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
// P*X of nvec vectors (stride N) at once, vector v with its own kernel shift
// e0v[v] (device): the level-1 matrices are staged once per block for all the
// vectors, and the outer rotations fold the vectors into the GEMM rows.
template <class T>
int px_multi(const scalit_ctx *c, const T *X, T *Y, T *tmp, int nvec, const double *e0v, const int *gate,
             cudaStream_t s, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
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
