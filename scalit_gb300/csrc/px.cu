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
// plus two n-vectors.
template <class T>
__global__ void __launch_bounds__(256)
px_level1_fused(int n, i64 nblk, const T *__restrict__ V, const T *__restrict__ EIG,
                const T *__restrict__ X, T *__restrict__ Y, KernelParams kp, T alpha,
                int v_in_smem, const int *gate)
{
    if (gate && *gate) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    T *ts = xs + n;
    T *Vs = ts + n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
    const T e0 = T(kp.e0), de = T(fabs(kp.de)), rde = T(1.0 / fabs(kp.de));
    const T beta_d = T(1.0 + kp.beta), alpha_d = T(-kp.beta * fabs(kp.de));

    for (i64 b = blockIdx.x; b < nblk; b += gridDim.x) {
        const T *Vb = V + b * (i64)n * n;
        const T *xb = X + b * (i64)n;
        __syncthreads();
        for (int i = tid; i < n; i += nt) xs[i] = xb[i];
        const T *Vsrc = Vb;
        if (v_in_smem) {
            const i64 nn = (i64)n * n;
            for (i64 e = tid; e < nn; e += nt) Vs[e] = Vb[e];
            Vsrc = Vs;
        }
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
            Y[b * (i64)n + i] = alpha * acc;
        }
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

template <class T>
static int launch_px1(int n, i64 nblk, const T *V, const T *EIG, const T *X, T *Y,
                      KernelParams kp, T alpha, const int *gate, cudaStream_t s)
{
    const size_t vec = sizeof(T) * 2 * (size_t)n;
    const size_t mat = sizeof(T) * (size_t)n * n;
    const int v_in_smem = (vec + mat <= kMaxDynSmem) ? 1 : 0;
    const size_t sm = vec + (v_in_smem ? mat : 0);
    static bool configured[2] = {false, false};
    const int which = sizeof(T) == 8 ? 0 : 1;
    if (!configured[which]) {
        SC_CUDA(cudaFuncSetAttribute(px_level1_fused<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kMaxDynSmem));
        configured[which] = true;
    }
    px_level1_fused<T><<<grid_for(nblk), 256, sm, s>>>(n, nblk, V, EIG, X, Y, kp, alpha, v_in_smem, gate);
    SC_CHECK_LAUNCH();
    return 0;
}

template <class T> static const T *pickp(const double *d, const float *f);
template <> const double *pickp<double>(const double *d, const float *) { return d; }
template <> const float *pickp<float>(const double *, const float *f) { return f; }

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
        rc = level_rotate<T>((int)L.dim[l], L.n[l], (int)L.blk[l], V + L.vs[l], in, out, 1, gate, s);
        if (rc) return rc;
        in = out;
    }
    ++stage;
    {
        T *out = buf[(S - stage) % 2];
        rc = launch_px1<T>(L.n[0], L.blk[0], V + L.vs[0], EIG, in, out, kp, alpha, gate, s);
        if (rc) return rc;
        in = out;
    }
    for (int l = 1; l < L.nlev; ++l) {
        ++stage;
        T *out = buf[(S - stage) % 2];
        rc = level_rotate<T>((int)L.dim[l], L.n[l], (int)L.blk[l], V + L.vs[l], in, out, 0, gate, s);
        if (rc) return rc;
        in = out;
    }
    return 0;
}

template int px_vec<double>(const scalit_ctx *, int, const double *, double *, double *, double, const int *, cudaStream_t);
template int px_vec<float>(const scalit_ctx *, int, const float *, float *, float *, float, const int *, cudaStream_t);

}  // namespace sc
