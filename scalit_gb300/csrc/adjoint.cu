// Adjoint of the H*X product and Hellmann-Feynman eigenvalue gradients.
//
// For Y = (V - E0) .* X + sum_l H_l X  (MYHX, src/iterate/module/osb.hx.h:71-110)
// and a cotangent Ybar:
//   Xbar  = (V - E0) .* Ybar + sum_l H_l^T Ybar        (the level matrices transposed)
//   Vbar  = Ybar .* X
//   Hbar_l(i, j) = sum_{a,b} s_l(a) Ybar(a, i, b) X(a, j, b)   (s_l = DEP of a dependent level)
// Hbar_l is a GEMM whose inner dimension is the whole grid except level l; it
// is split over the blocks b (and over chunks of a when a single block is
// large) into partial matrices that a second kernel sums in a fixed order.
//
// Hellmann-Feynman: for an eigenvector psi_k of H,  dE_k/dp = <psi_k| dV/dp |psi_k>
// = sum_p psi_k(p)^2 dV/dp(p) -- one deterministic reduction per (k, parameter).
#include "internal.cuh"

#include <algorithm>
#include <vector>

namespace sc {

template <class T>
__global__ void mul_kernel(i64 n, const T *__restrict__ a, const T *__restrict__ b, T *__restrict__ out,
                           int accumulate)
{
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const T v = a[i] * b[i];
        out[i] = accumulate ? out[i] + v : v;
    }
}

// out(a, i, b) = s(a) y(a, i, b) for a dependent level (a = fastest index, nin long)
template <class T>
__global__ void rowscale_kernel(i64 n, i64 nin, const T *__restrict__ s, const T *__restrict__ y, T *__restrict__ out)
{
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        out[i] = s[i % nin] * y[i];
}

// dst[e] (+)= sum_z partial[z][e], z in order
template <class T>
__global__ void sum_partials_kernel(int nz, i64 len, const T *__restrict__ partial, T *__restrict__ dst, int accumulate)
{
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < len; e += (i64)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int z = 0; z < nz; ++z) s += partial[(i64)z * len + e];
        dst[e] = accumulate ? dst[e] + s : s;
    }
}

template <class T>
__global__ void transpose_kernel(int n, const T *__restrict__ a, T *__restrict__ at)
{
    const i64 nn = (i64)n * n;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < nn; e += (i64)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        at[j + (i64)n * i] = a[e];
    }
}

static int egrid(i64 n)
{
    i64 g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    return (int)std::max<i64>(g, 1);
}

template <class T> static const T *pickd(const double *d, const float *f);
template <> const double *pickd<double>(const double *d, const float *) { return d; }
template <> const float *pickd<float>(const double *, const float *f) { return f; }

template <class T>
int hx_adjoint(scalit_ctx *c, int ntype, const T *X, const T *Ybar, T *Xbar, T *Vbar, T *Hbar, cudaStream_t s)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    const T *H0 = pickd<T>(c->H0, c->H0f);
    const T *RES = pickd<T>(c->RES, c->RESf);
    const T *DEP = pickd<T>(c->DEP, c->DEPf);
    const T shift = (ntype == SCALIT_TA0) ? T(0) : T(c->E0);
    if (L.ndvr) { set_error("the adjoint of the per-point outer layer is not provided"); return SCALIT_EUNSUP; }
    int rc = 0;
    if (Xbar) {
        // transposed level matrices, then the forward operator
        T *H0T = nullptr;
        SC_CUDA(cudaMallocAsync(&H0T, sizeof(T) * (size_t)std::max<i64>(L.h0len, 1), s));
        for (int l = 0; l < L.nlev; ++l)
            transpose_kernel<T><<<egrid((i64)L.n[l] * L.n[l]), 256, 0, s>>>(L.n[l], H0 + L.h0s[l], H0T + L.h0s[l]);
        SC_CHECK_LAUNCH();
        for (int l = 0; l < L.nlev && !rc; ++l)
            rc = level_apply<T>(c, l, H0T, DEP, nullptr, Ybar, Xbar, l > 0, l == 0 ? RES : nullptr, shift, T(1),
                                nullptr, s, 1);
        cudaFreeAsync(H0T, s);
        if (rc) return rc;
    }
    if (Vbar) {
        mul_kernel<T><<<egrid(N), 256, 0, s>>>(N, Ybar, X, Vbar, 0);
        SC_CHECK_LAUNCH();
    }
    if (Hbar) {
        T *ys = nullptr;
        SC_CUDA(cudaMallocAsync(&ys, sizeof(T) * (size_t)N, s));
        for (int l = 0; l < L.nlev && !rc; ++l) {
            const int nout = L.n[l];
            const i64 nin = L.dim[l], blk = L.blk[l];
            const T *Y = Ybar;
            if (L.dep[l]) {
                rowscale_kernel<T><<<egrid(N), 256, 0, s>>>(N, nin, DEP + L.deps[l], Ybar, ys);
                Y = ys;
            }
            if (nin == 1) {
                // Hbar(i, j) = sum_b Y(i, b) X(j, b): one long inner dimension, split into
                // chunks of kc blocks (the last one shorter), summed in chunk order
                const i64 kc = 4096, nch = (blk + kc - 1) / kc, nfull = blk / kc;
                T *part = nullptr;
                SC_CUDA(cudaMallocAsync(&part, sizeof(T) * (size_t)(nch * nout * nout), s));
                for (int pass = 0; pass < 2 && !rc; ++pass) {
                    const i64 z0 = pass ? nfull : 0, nzb = pass ? nch - nfull : nfull;
                    if (nzb <= 0) continue;
                    GemmArgs<T> g{};
                    g.M = nout; g.N = nout; g.K = (int)(pass ? blk - nfull * kc : kc);
                    g.batch = (int)nzb;
                    g.Mi = nout; g.s1 = 1; g.s2 = 0;
                    g.A = Y + z0 * kc * nout; g.a_sk = nout; g.a_sz = kc * nout;     // A(i, b) = Y[i + nout b]
                    g.B = X + z0 * kc * nout; g.b_sk = nout; g.b_sn = 1; g.b_sz = kc * nout;   // B(b, j) = X[j + nout b]
                    g.C = part + z0 * nout * nout; g.c_sn = nout; g.c_sz = (i64)nout * nout;
                    g.alpha = T(1);
                    rc = launch_gemm<T>(g, s);
                }
                if (!rc) {
                    sum_partials_kernel<T><<<egrid((i64)nout * nout), 256, 0, s>>>((int)nch, (i64)nout * nout, part,
                                                                                   Hbar + L.h0s[l], 0);
                    if (cudaGetLastError() != cudaSuccess) { set_error("partial sum launch"); rc = SCALIT_ECUDA; }
                }
                cudaFreeAsync(part, s);
                continue;
            }
            // split the inner dimension (a over nin, b over blk) into nz pieces of kc points of a
            const i64 kc = std::min<i64>(nin, 4096);
            const i64 nchunk = (nin + kc - 1) / kc;
            const i64 nz = nchunk * blk;
            T *part = nullptr;
            SC_CUDA(cudaMallocAsync(&part, sizeof(T) * (size_t)(nz * nout * nout), s));
            SC_CUDA(cudaMemsetAsync(part, 0, sizeof(T) * (size_t)(nz * nout * nout), s));
            for (i64 ch = 0; ch < nchunk && !rc; ++ch) {
                const i64 a0 = ch * kc, ka = std::min(kc, nin - a0);
                // partial_{ch,b}(i, j) = sum_{a in chunk} Y(a, i, b) X(a, j, b)
                GemmArgs<T> g{};
                g.M = nout; g.N = nout; g.K = (int)ka;
                g.batch = (int)blk;
                g.Mi = nout; g.s1 = nin; g.s2 = 0;           // A(i, a) = Y[a + nin i]
                g.c_s1 = 1; g.c_s2 = 0;                      // C(i, j) = part[i + nout j]
                g.A = Y + a0; g.a_sk = 1; g.a_sz = nin * nout;
                g.B = X + a0; g.b_sk = 1; g.b_sn = nin; g.b_sz = nin * nout;   // B(a, j) = X[a + nin j]
                g.C = part + ch * blk * (i64)nout * nout; g.c_sn = nout; g.c_sz = (i64)nout * nout;
                g.alpha = T(1);
                if (blk > 65535) {
                    for (i64 b0 = 0; b0 < blk && !rc; b0 += 65535) {
                        GemmArgs<T> h = g;
                        h.batch = (int)std::min<i64>(65535, blk - b0);
                        h.A = g.A + b0 * nin * nout;
                        h.B = g.B + b0 * nin * nout;
                        h.C = g.C + b0 * (i64)nout * nout;
                        rc = launch_gemm<T>(h, s);
                    }
                } else {
                    rc = launch_gemm<T>(g, s);
                }
            }
            if (!rc) {
                sum_partials_kernel<T><<<egrid((i64)nout * nout), 256, 0, s>>>((int)nz, (i64)nout * nout, part,
                                                                               Hbar + L.h0s[l], 0);
                if (cudaGetLastError() != cudaSuccess) { set_error("partial sum launch"); rc = SCALIT_ECUDA; }
            }
            cudaFreeAsync(part, s);
        }
        cudaFreeAsync(ys, s);
    }
    return rc;
}

template int hx_adjoint<double>(scalit_ctx *, int, const double *, const double *, double *, double *, double *, cudaStream_t);
template int hx_adjoint<float>(scalit_ctx *, int, const float *, const float *, float *, float *, float *, cudaStream_t);

// grad[k * np + j] = sum_p psi_k(p)^2 dvdp_j(p)
__global__ void __launch_bounds__(256)
hf_kernel(i64 n, int m, int np, const double *__restrict__ psi, const double *__restrict__ dvdp,
          double *__restrict__ partial)
{
    const int k = blockIdx.y / np, j = blockIdx.y % np;
    const double *u = psi + (i64)k * n;
    const double *d = dvdp + (i64)j * n;
    double a = 0.0;
    for (i64 p = blockIdx.x * (i64)blockDim.x + threadIdx.x; p < n; p += (i64)gridDim.x * blockDim.x)
        a = fma(u[p] * u[p], d[p], a);
    __shared__ double red[8];
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += red[w];
        partial[(i64)blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
    (void)m;
}

__global__ void hf_fold_kernel(int nk, int nchunk, const double *partial, double *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nk) return;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += partial[(i64)e * nchunk + c];
    out[e] = s;
}

int hf_gradients(scalit_ctx *c, int m, const double *psi, int np, const double *dvdp, double *grad_dev)
{
    const i64 n = c->L.N;
    const int nchunk = 64;
    if ((i64)m * np > 65535) { set_error("too many (level, parameter) pairs"); return SCALIT_EINVAL; }
    double *partial = nullptr;
    cudaStream_t s = c->stream;
    SC_CUDA(cudaMallocAsync(&partial, sizeof(double) * (size_t)m * np * nchunk, s));
    hf_kernel<<<dim3(nchunk, m * np), 256, 0, s>>>(n, m, np, psi, dvdp, partial);
    hf_fold_kernel<<<(m * np + 127) / 128, 128, 0, s>>>(m * np, nchunk, partial, grad_dev);
    SC_CHECK_LAUNCH();
    cudaFreeAsync(partial, s);
    return 0;
}

}  // namespace sc
