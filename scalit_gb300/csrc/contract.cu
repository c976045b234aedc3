// Per-level contractions of the H*X product and of the preconditioner
// rotations, as one strided tiled GEMM kernel.
//
// Every level of MYHX (src/iterate/module/osb.hx.h:71-110) is a GEMM once the
// grid vector is viewed through the level's strides:
//   level with nin == 1   : Y(i, b)        = sum_j H(i, j) X(j, b)          (H1X, nin = 1)
//   level with nin  > 1   : Y(a, i, b)     = s(a) sum_j H(i, j) X(a, j, b)   (H1X / H2X)
// The first is C = H * X (M = nout, N = blk), the second folds (a, b) into M
// (M = nin*blk, N = nout) with H^T as the B operand.  The diagonal potential
// term of MYHX is fused into the epilogue of the first level.
//
// FP64 tiles are 64x64x16 with 4x4 outputs per thread, FP32 tiles 128x128x8
// with 8x8 outputs per thread; A and B tiles are staged k-major in shared
// memory with a register prefetch of the next K slab.
#include "internal.cuh"

#include <type_traits>

namespace sc {

// Tile shapes: 256 threads, TM x TN outputs per thread.  The small tiles are
// used when the large ones would give the launch fewer than about three waves
// of CTAs on the 152 SMs (a single-vector level has only a few hundred tiles).
template <int BM_, int BN_, int BK_, int TM_, int TN_> struct TileCfg {
    static constexpr int BM = BM_, BN = BN_, BK = BK_, TM = TM_, TN = TN_;
};
template <class T> struct Tiles;
template <> struct Tiles<double> { using Big = TileCfg<64, 64, 16, 4, 4>; using Small = TileCfg<32, 32, 16, 2, 2>; };
template <> struct Tiles<float> { using Big = TileCfg<128, 128, 8, 8, 8>; using Small = TileCfg<64, 64, 8, 4, 4>; };

template <class T, class TL>
__global__ void __launch_bounds__(256)
gemm_kernel(GemmArgs<T> g)
{
    constexpr int BM = TL::BM, BN = TL::BN, BK = TL::BK, TM = TL::TM, TN = TL::TN;
    constexpr int NT = 256;
    constexpr int A_PER = BM * BK / NT;   // A elements each thread loads per slab
    constexpr int B_PER = BN * BK / NT;
    static_assert((BM / TM) * (BN / TN) == NT, "thread grid");

    if (g.gate && *g.gate) return;
    if (g.vgate && g.vgate[(i64)(blockIdx.z / g.vgate_div) * g.vgate_stride]) return;

    __shared__ T As[BK][BM];
    __shared__ T Bs[BK][BN];

    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int z = blockIdx.z;
    const T *A = g.A + (i64)z * g.a_sz;
    const T *B = g.B + (i64)(g.b_mod > 0 ? z % g.b_mod : z) * g.b_sz;
    T *Cp = g.C + (i64)z * g.c_sz;

    // Loader mapping.  A: consecutive threads take consecutive m (coalesced
    // along the contiguous grid axis).  B: consecutive threads take
    // consecutive n when B's n-stride is 1, else consecutive k.
    const bool b_n_fast = (g.b_sn == 1);
    i64 a_moff[A_PER];
    int a_m[A_PER], a_k[A_PER];
    #pragma unroll
    for (int r = 0; r < A_PER; ++r) {
        const int e = tid + r * NT;
        a_m[r] = e % BM;
        a_k[r] = e / BM;
        const int m = m0 + a_m[r];
        a_moff[r] = (m < g.M) ? ((i64)(m % g.Mi) * g.s1 + (i64)(m / g.Mi) * g.s2) : -1;
    }
    int b_n[B_PER], b_k[B_PER];
    #pragma unroll
    for (int r = 0; r < B_PER; ++r) {
        const int e = tid + r * NT;
        if (b_n_fast) { b_n[r] = e % BN; b_k[r] = e / BN; }
        else { b_k[r] = e % BK; b_n[r] = e / BK; }
    }

    T ra[A_PER], rb[B_PER];
    auto load = [&](int k0) {
        #pragma unroll
        for (int r = 0; r < A_PER; ++r) {
            const int k = k0 + a_k[r];
            ra[r] = (a_moff[r] >= 0 && k < g.K) ? A[a_moff[r] + (i64)k * g.a_sk] : T(0);
        }
        #pragma unroll
        for (int r = 0; r < B_PER; ++r) {
            const int k = k0 + b_k[r], n = n0 + b_n[r];
            rb[r] = (k < g.K && n < g.N) ? B[(i64)k * g.b_sk + (i64)n * g.b_sn] : T(0);
        }
    };
    auto store = [&]() {
        #pragma unroll
        for (int r = 0; r < A_PER; ++r) As[a_k[r]][a_m[r]] = ra[r];
        #pragma unroll
        for (int r = 0; r < B_PER; ++r) Bs[b_k[r]][b_n[r]] = rb[r];
    };

    const int tm = (tid % (BM / TM)) * TM;   // this thread's rows within the tile
    const int tn = (tid / (BM / TM)) * TN;   // this thread's columns
    T acc[TM][TN];
    #pragma unroll
    for (int i = 0; i < TM; ++i)
        #pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

    load(0);
    for (int k0 = 0; k0 < g.K; k0 += BK) {
        __syncthreads();
        store();
        __syncthreads();
        if (k0 + BK < g.K) load(k0 + BK);
        #pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T av[TM], bv[TN];
            #pragma unroll
            for (int i = 0; i < TM; ++i) av[i] = As[kk][tm + i];
            #pragma unroll
            for (int j = 0; j < TN; ++j) bv[j] = Bs[kk][tn + j];
            #pragma unroll
            for (int i = 0; i < TM; ++i)
                #pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
    }

    // Epilogue: every load (diagonal, accumulated output) before any store, so
    // the thread's TM x TN loads are in flight together instead of one
    // round trip per output (a store to C could alias a later load).
    const i64 cs1 = g.c_s1 >= 0 ? g.c_s1 : g.s1, cs2 = g.c_s2 >= 0 ? g.c_s2 : g.s2;
    i64 moffs[TM];
    #pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int m = m0 + tm + i;
        const i64 mi = m < g.M ? m % g.Mi : 0;
        moffs[i] = mi * cs1 + (i64)(m < g.M ? m / g.Mi : 0) * cs2;
        const T sc = g.rowscale ? g.rowscale[mi] * g.alpha : g.alpha;
        #pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + tn + j;
            if (m >= g.M || n >= g.N) continue;
            const i64 p = moffs[i] + (i64)n * g.c_sn;
            T v = sc * acc[i][j];
            if (g.diagV) v = fma(g.alpha * (g.diagV[p] - (g.shiftv ? g.shiftv[z] : g.shift)), g.diagX[p + (i64)z * g.dx_sz], v);
            if (g.accumulate) v += Cp[p];
            acc[i][j] = v;
        }
    }
    #pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int m = m0 + tm + i;
        #pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n0 + tn + j;
            if (m >= g.M || n >= g.N) continue;
            Cp[moffs[i] + (i64)n * g.c_sn] = acc[i][j];
        }
    }
}

template <class T, class TL> static int launch_tiles(const GemmArgs<T> &g, cudaStream_t s)
{
    dim3 grid((g.M + TL::BM - 1) / TL::BM, (g.N + TL::BN - 1) / TL::BN, g.batch);
    if (grid.y > 65535) { set_error("gemm N=%d too large", g.N); return SCALIT_EINVAL; }
    gemm_kernel<T, TL><<<grid, 256, 0, s>>>(g);
    SC_CHECK_LAUNCH();
    return 0;
}

template <class T> int launch_gemm(const GemmArgs<T> &g, cudaStream_t s)
{
    using Big = typename Tiles<T>::Big;
    using Small = typename Tiles<T>::Small;
    if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return 0;
    if (g.batch > 65535) { set_error("gemm batch %d too large", g.batch); return SCALIT_EINVAL; }
    if (g.tile == 0) return launch_tiles<T, Big>(g, s);
    if (g.tile == 1) return launch_tiles<T, Small>(g, s);
    // untuned: the small tile unless the big one fills the GPU three times
    const i64 big_ctas = (i64)((g.M + Big::BM - 1) / Big::BM) * ((g.N + Big::BN - 1) / Big::BN) * g.batch;
    if (big_ctas < 3 * 2 * 152) return launch_tiles<T, Small>(g, s);
    return launch_tiles<T, Big>(g, s);
}

template int launch_gemm<double>(const GemmArgs<double> &, cudaStream_t);
template int launch_gemm<float>(const GemmArgs<float> &, cudaStream_t);

// ------------------------------------------------------------------------
// H3X (src/libutil/serial/base/matrix.f90:188-203): outermost layer given as
// per-point matrices A(nin, nout, nout): Y(a, i) (+)= sum_j A(a, i, j) X(a, j).
template <class T>
__global__ void h3x_kernel(int nin, int nout, const T *__restrict__ Am, const T *__restrict__ X,
                           T *__restrict__ Y, int accumulate, T alpha, const int *gate)
{
    if (gate && *gate) return;
    const i64 total = (i64)nin * nout;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
         e += (i64)gridDim.x * blockDim.x) {
        const i64 a = e % nin;
        const int i = (int)(e / nin);
        T acc = T(0);
        for (int j = 0; j < nout; ++j)
            acc = fma(Am[a + (i64)nin * (i + (i64)nout * j)], X[a + (i64)nin * j], acc);
        const T v = alpha * acc;
        Y[e] = accumulate ? Y[e] + v : v;
    }
}

template <class T>
int level_apply(const scalit_ctx *c, int l, const T *H0, const T *DEP, const T *OUTH, const T *X,
                T *Y, int accumulate, const T *diagV, T shift, T alpha, const int *gate,
                cudaStream_t s, int nvec, const T *shiftv, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const int nout = L.n[l];
    const i64 nin = L.dim[l], blk = L.blk[l], N = L.N;
    if (nvec < 1) return 0;
    if (L.ndvr && l == L.nlev - 1) {
        // Outer per-point matrices; the diagonal term, if requested, is a
        // separate pass (the outermost level is never the first applied).
        if (diagV) { set_error("diagonal fused into the outer layer"); return SCALIT_EINVAL; }
        const i64 total = nin * nout;
        const int threads = 256;
        const int blocks = (int)((total + threads - 1) / threads < 152 * 16 ? (total + threads - 1) / threads : 152 * 16);
        for (int v = 0; v < nvec; ++v) {
            h3x_kernel<T><<<blocks, threads, 0, s>>>((int)nin, nout, OUTH, X + (i64)v * N, Y + (i64)v * N,
                                                     accumulate, alpha, gate);
            SC_CHECK_LAUNCH();
        }
        return 0;
    }
    GemmArgs<T> g{};
    g.K = nout;
    g.batch = nvec;
    g.accumulate = accumulate;
    g.alpha = alpha;
    g.diagV = diagV;
    g.diagX = X;
    g.dx_sz = N;
    g.shift = shift;
    g.shiftv = shiftv;
    g.gate = gate;
    g.C = Y;
    g.c_sz = N;
    g.tile = c->tile_pick[sizeof(T) == 8 ? 0 : 1][l][nvec > 1 ? 1 : 0];
    g.vgate = vgate;
    g.vgate_stride = vstride;
    const T *H = H0 + L.h0s[l];
    if (nin == 1) {
        // Y(i, b) = sum_j H(i, j) X(j, b): A = H (col-major), B = X.
        g.M = nout; g.N = (int)blk;
        g.Mi = nout; g.s1 = 1; g.s2 = 0;
        g.A = H; g.a_sk = nout; g.a_sz = 0;
        g.B = X; g.b_sk = 1; g.b_sn = nout; g.b_sz = N;
        g.c_sn = nout;
        g.rowscale = nullptr;
        if (blk > 65535LL * Tiles<T>::Small::BN) { set_error("level %d too many blocks", l + 1); return SCALIT_EINVAL; }
    } else {
        // Y(a, i, b) = s(a) sum_j X(a, j, b) H(i, j): A = X with (a, b) folded, B = H^T.
        const i64 M = nin * blk;
        if (M > 2147483647LL) { set_error("level %d too large", l + 1); return SCALIT_EINVAL; }
        g.M = (int)M; g.N = nout;
        g.Mi = nin; g.s1 = 1; g.s2 = nin * nout;
        g.A = X; g.a_sk = nin; g.a_sz = N;
        g.B = H; g.b_sk = nout; g.b_sn = 1; g.b_sz = 0;
        g.c_sn = nin;
        g.rowscale = L.dep[l] ? DEP + L.deps[l] : nullptr;
    }
    return launch_gemm<T>(g, s);
}

template <class T>
__global__ void diag_kernel(i64 n, const T *__restrict__ V, T shift, T alpha,
                            const T *__restrict__ X, T *__restrict__ Y, int accumulate,
                            const int *gate)
{
    if (gate && *gate) return;
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const T v = alpha * (V[i] - shift) * X[i];
        Y[i] = accumulate ? Y[i] + v : v;
    }
}

template <class T> static const T *pick(const scalit_ctx *c, const double *d, const float *f);
template <> const double *pick<double>(const scalit_ctx *, const double *d, const float *) { return d; }
template <> const float *pick<float>(const scalit_ctx *, const double *, const float *f) { return f; }

template <class T>
int hx_batch(const scalit_ctx *c, const T *X, T *Y, int nvec, T shift, T alpha, const int *gate,
             cudaStream_t s, const T *shiftv, const int *vgate, int vstride)
{
    const Layout &L = c->L;
    const T *H0 = pick<T>(c, c->H0, c->H0f);
    const T *RES = pick<T>(c, c->RES, c->RESf);
    const T *DEP = pick<T>(c, c->DEP, c->DEPf);
    const T *OUTH = pick<T>(c, c->OUTH, c->OUTHf);
    int rc;
    int first = 0;
    // FP32 tensor-core forms: the persistent pipelined level kernel wherever
    // it applies (split-FP16 x3 needs the vectors' scales first)
    bool p16 = false, pbf = false, p64 = false;
    if constexpr (std::is_same<T, double>::value) {
        // FP64 digit engine: the persistent kernel wherever it applies, after
        // the vectors' exponents
        const bool aligned = !(reinterpret_cast<uintptr_t>(X) & 15) && !(reinterpret_cast<uintptr_t>(Y) & 15);
        if (aligned && c->fp64_mode == SCALIT_FP64_TENSOR && nvec <= tc64p_vectors_max()) {
            for (int l = 0; l < L.nlev; ++l) {
                if (!tc64p_usable(c, l)) continue;
                p64 = true;
                rc = tc64p_rowexp(c, l, X, nvec, gate, s, vgate, vstride);
                if (rc) return rc;
            }
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        const bool aligned = !(reinterpret_cast<uintptr_t>(X) & 15) && !(reinterpret_cast<uintptr_t>(Y) & 15);
        p16 = aligned && c->fp32_mode == SCALIT_FP32_TENSOR16;
        pbf = aligned && c->fp32_mode == SCALIT_FP32_TENSOR;
        bool any16 = false;
        for (int l = 0; l < L.nlev && p16; ++l) any16 = any16 || tc32p_usable(c, l, true);
        if (any16) {
            rc = tc16_scales(c, X, nvec, gate, s, vgate, vstride);
            if (rc) return rc;
        } else {
            p16 = false;
        }
    }
    // The diagonal term rides on the first level's epilogue, except on the
    // persistent kernel: there the last level (grid points contiguous per
    // column, its output already read for the accumulation) takes it, so the
    // first level's epilogue loads nothing.
    int diag_level = 0;
    if ((p16 || pbf) && L.nlev > 1 && tc32p_usable(c, L.nlev - 1, p16, true)) diag_level = L.nlev - 1;
    if (p64 && L.nlev > 1 && tc64p_usable(c, L.nlev - 1)) diag_level = L.nlev - 1;
    if (L.ndvr && L.nlev == 1) {
        const int threads = 256;
        if (shiftv) { set_error("per-vector shifts with a single outer layer"); return SCALIT_EUNSUP; }
        for (int v = 0; v < nvec; ++v) {
            diag_kernel<T><<<(int)((L.N + threads - 1) / threads), threads, 0, s>>>(
                L.N, RES, shift, alpha, X + (i64)v * L.N, Y + (i64)v * L.N, 0, gate);
            SC_CHECK_LAUNCH();
        }
        first = 1;
    }
    for (int l = 0; l < L.nlev; ++l) {
        if (c->lev_ev) cudaEventRecord(c->lev_ev[l], s);
        const bool fuse_diag = (l == diag_level && !first);
        if constexpr (std::is_same<T, double>::value) {
            if (p64 && tc64p_usable(c, l)) {
                rc = tc64p_level_apply(c, l, X, Y, l > 0 || first, fuse_diag ? RES : nullptr, shift, alpha,
                                       gate, s, nvec, shiftv, vgate, vstride);
                if (rc) return rc;
                continue;
            }
            if (c->fp64_mode == SCALIT_FP64_TENSOR && tc_usable(c, l)) {
                rc = tc_level_apply(c, l, X, Y, l > 0 || first, fuse_diag ? RES : nullptr, shift, alpha,
                                    gate, s, nvec, shiftv, vgate, vstride);
                if (rc) return rc;
                continue;
            }
        } else {
            if ((p16 || pbf) && tc32p_usable(c, l, p16, fuse_diag)) {
                rc = tc32p_level_apply(c, l, p16, X, Y, l > 0 || first, fuse_diag ? RES : nullptr, shift, alpha,
                                       gate, s, nvec, shiftv, vgate, vstride);
                if (rc) return rc;
                continue;
            }
            if (tc32_usable(c, l)) {
                rc = tc32_level_apply(c, l, X, Y, l > 0 || first, fuse_diag ? RES : nullptr, shift, alpha,
                                      gate, s, nvec, shiftv, vgate, vstride);
                if (rc) return rc;
                continue;
            }
        }
        rc = level_apply<T>(c, l, H0, DEP, OUTH, X, Y, /*accumulate=*/l > 0 || first,
                            fuse_diag ? RES : nullptr, shift, alpha, gate, s, nvec, shiftv, vgate, vstride);
        if (rc) return rc;
    }
    if (c->lev_ev) cudaEventRecord(c->lev_ev[L.nlev], s);
    return 0;
}

template <class T>
int hx_vec(const scalit_ctx *c, const T *X, T *Y, T shift, T alpha, const int *gate, cudaStream_t s)
{
    return hx_batch<T>(c, X, Y, 1, shift, alpha, gate, s);
}

template int hx_batch<double>(const scalit_ctx *, const double *, double *, int, double, double, const int *, cudaStream_t, const double *, const int *, int);
template int hx_batch<float>(const scalit_ctx *, const float *, float *, int, float, float, const int *, cudaStream_t, const float *, const int *, int);
template int hx_vec<double>(const scalit_ctx *, const double *, double *, double, double, const int *, cudaStream_t);
template int hx_vec<float>(const scalit_ctx *, const float *, float *, float, float, const int *, cudaStream_t);
template int level_apply<double>(const scalit_ctx *, int, const double *, const double *, const double *, const double *, double *, int, const double *, double, double, const int *, cudaStream_t, int, const double *, const int *, int);
template int level_apply<float>(const scalit_ctx *, int, const float *, const float *, const float *, const float *, float *, int, const float *, float, float, const int *, cudaStream_t, int, const float *, const int *, int);

// ------------------------------------------------------------------------
// VX / VTX (src/iterate/libiterate/hpx/hpx.f90:40-73) out of place:
// Y(:, i, b) = sum_j V(i, j, b) X(:, j, b)  (VX)   or  sum_j V(j, i, b) X(:, j, b)  (VTX).
template <class T>
int bgemv(int nout, int blk, const T *V, const T *X, T *Y, int transpose, const int *gate,
          cudaStream_t s);

template <class T>
int level_rotate(int nin, int nout, int blk, const T *V, const T *X, T *Y, int transpose,
                 const int *gate, cudaStream_t s)
{
    GemmArgs<T> g{};
    g.K = nout;
    g.accumulate = 0;
    g.alpha = T(1);
    g.gate = gate;
    g.rowscale = nullptr;
    g.diagV = nullptr;
    g.C = Y;
    if (nin == 1) return bgemv(nout, blk, V, X, Y, transpose, gate, s);
    // per block b: Y_b(a, i) = sum_j X_b(a, j) V_b(i, j)  -> A = X_b, B = V_b^T (VX) or V_b (VTX)
    g.M = nin; g.N = nout; g.batch = blk;
    g.Mi = nin; g.s1 = 1; g.s2 = 0;
    g.A = X; g.a_sk = nin; g.a_sz = (i64)nin * nout;
    g.B = V; g.b_sz = (i64)nout * nout;
    if (!transpose) { g.b_sk = nout; g.b_sn = 1; }
    else { g.b_sk = 1; g.b_sn = nout; }
    g.c_sn = nin; g.c_sz = (i64)nin * nout;
    return launch_gemm<T>(g, s);
}

template int level_rotate<double>(int, int, int, const double *, const double *, double *, int, const int *, cudaStream_t);
// Tile autotuner: for every level, both precisions of the CUDA-core GEMM and
// one or many vectors, time the big and the small tile on the level's own
// shapes (two launches each after one warm-up, CUDA events) and keep the
// faster.  Scratch comes from the context's workspace.
template <class T>
static int tune_one(scalit_ctx *c, int l, int nvec, T *X, T *Y, cudaEvent_t e0, cudaEvent_t e1)
{
    const T *H0 = (sizeof(T) == 8) ? (const T *)c->H0 : (const T *)c->H0f;
    const T *DEP = (sizeof(T) == 8) ? (const T *)c->DEP : (const T *)c->DEPf;
    const T *OUTH = (sizeof(T) == 8) ? (const T *)c->OUTH : (const T *)c->OUTHf;
    cudaStream_t s = c->stream;
    float best = 0.f;
    int pick = -1;
    for (int tile = 0; tile < 2; ++tile) {
        c->tile_pick[sizeof(T) == 8 ? 0 : 1][l][nvec > 1 ? 1 : 0] = (signed char)tile;
        int rc = level_apply<T>(c, l, H0, DEP, OUTH, X, Y, 0, nullptr, T(0), T(1), nullptr, s, nvec);
        if (rc) return rc;
        SC_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 2 && !rc; ++r)
            rc = level_apply<T>(c, l, H0, DEP, OUTH, X, Y, 0, nullptr, T(0), T(1), nullptr, s, nvec);
        if (rc) return rc;
        SC_CUDA(cudaEventRecord(e1, s));
        SC_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (pick < 0 || ms < best) { best = ms; pick = tile; }
    }
    c->tile_pick[sizeof(T) == 8 ? 0 : 1][l][nvec > 1 ? 1 : 0] = (signed char)pick;
    return 0;
}

int gemm_autotune(scalit_ctx *c, int nvec_many)
{
    const Layout &L = c->L;
    const i64 N = L.N;
    if (nvec_many < 2) nvec_many = 2;
    void *w = nullptr;
    int rc = work_get(c, sizeof(double) * 2 * (size_t)N * nvec_many, &w);
    if (rc) return rc;
    SC_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * 2 * (size_t)N * nvec_many, c->stream));
    cudaEvent_t e0, e1;
    SC_CUDA(cudaEventCreate(&e0));
    SC_CUDA(cudaEventCreate(&e1));
    for (int l = 0; l < L.nlev && !rc; ++l) {
        if (L.ndvr && l == L.nlev - 1) continue;
        for (int many = 0; many < 2 && !rc; ++many) {
            const int nv = many ? nvec_many : 1;
            double *X64 = reinterpret_cast<double *>(w), *Y64 = X64 + (size_t)N * nv;
            float *X32 = reinterpret_cast<float *>(w), *Y32 = X32 + (size_t)N * nv;
            // the FP64 CUDA-core GEMM serves single vectors in the bit-reproducible mode
            if (!many) rc = tune_one<double>(c, l, nv, X64, Y64, e0, e1);
            if (!rc) rc = tune_one<float>(c, l, nv, X32, Y32, e0, e1);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}


template int level_rotate<float>(int, int, int, const float *, const float *, float *, int, const int *, cudaStream_t);

}  // namespace sc
