// The C ABI of libscalit_gb300: context management, the whole-operator entry
// points and the Fortran drop-in symbols (gfortran naming, arguments by
// reference, caller-owned host arrays).
#include "internal.cuh"

#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <vector>

namespace sc {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line)
{
    set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    if (e == cudaErrorMemoryAllocation) return SCALIT_ENOMEM;
    return SCALIT_ECUDA;
}

void Layout::compute()
{
    dim[0] = 1;
    for (int i = 0; i < nlev - 1; ++i) dim[i + 1] = dim[i] * n[i];
    blk[nlev - 1] = 1;
    for (int i = nlev - 1; i >= 1; --i) blk[i - 1] = blk[i] * n[i];
    N = blk[0] * n[0];
    i64 h = 0, d = 0, v = 0;
    for (int i = 0; i < nlev; ++i) {
        h0s[i] = h;
        if (!(ndvr && i == nlev - 1)) h += (i64)n[i] * n[i];
        deps[i] = d;
        if (dep[i]) d += dim[i];
        vs[i] = v;
        v += blk[i] * (i64)n[i] * n[i];
    }
    h0len = h;
    deplen = d;
    vlen = v;
    outhlen = ndvr ? (i64)n[nlev - 1] * N : 0;
}

int work_get(scalit_ctx *c, size_t bytes, void **out)
{
    if (c->work_bytes < bytes) {
        if (c->work) {
            cudaStreamSynchronize(c->stream);
            cudaFree(c->work);
            c->work = nullptr;
            c->work_bytes = 0;
        }
        SC_CUDA(cudaMalloc(&c->work, bytes));
        c->work_bytes = bytes;
        c->gen++;
    }
    *out = c->work;
    return 0;
}

int sync_read_doubles(scalit_ctx *c, const double *dsrc, double *host, int count)
{
    SC_CUDA(cudaMemcpyAsync(c->h_pinned, dsrc, sizeof(double) * count, cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    memcpy(host, c->h_pinned, sizeof(double) * count);
    return 0;
}

// Scratch context for routines that need only a stream and reduction scratch.
static int ctx_base_init(scalit_ctx *c, int device)
{
    c->device = device;
    SC_CUDA(cudaSetDevice(device));
    SC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    SC_CUDA(cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking));
    SC_CUDA(cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking));
    for (int i = 0; i < 6; ++i) SC_CUDA(cudaEventCreateWithFlags(&c->ev[i], cudaEventDisableTiming));
    SC_CUDA(cudaMalloc(&c->red_partial, sizeof(double) * 4 * 152 * 4 + 64));
    SC_CUDA(cudaMalloc(&c->red_counter, sizeof(unsigned int) * 4));
    SC_CUDA(cudaMemset(c->red_counter, 0, sizeof(unsigned int) * 4));
    SC_CUDA(cudaMalloc(&c->red_result, sizeof(double) * 16));
    SC_CUDA(cudaMallocHost(&c->h_pinned, 4096));
    cusolverDnHandle_t h = nullptr;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnCreate failed");
        return SCALIT_ECUDA;
    }
    c->cusolver = h;
    return 0;
}

static bool all_finite(const double *a, i64 n)
{
    for (i64 i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

template <class T>
static int hx_many(scalit_ctx *c, int ntype, int nvec, const T *dX, T *dY)
{
    if (!c->loaded) { set_error("H*X before scalit_load"); return SCALIT_ESTATE; }
    if (nvec < 0) { set_error("nvec < 0"); return SCALIT_EINVAL; }
    if (ntype != SCALIT_TA0 && ntype != SCALIT_TA1) { set_error("ntype must be TA0 or TA1"); return SCALIT_EINVAL; }
    const T shift = ntype == SCALIT_TA0 ? T(0) : T(c->E0);
    const i64 N = c->L.N;
    // batches of at most 64 vectors per launch (grid z)
    for (int v = 0; v < nvec; v += 64) {
        const int nb = nvec - v < 64 ? nvec - v : 64;
        int rc = hx_batch<T>(c, dX + (i64)v * N, dY + (i64)v * N, nb, shift, T(1), nullptr, c->stream);
        if (rc) return rc;
    }
    return 0;
}

template <class T>
static int px_many(scalit_ctx *c, int npc, int nvec, const T *dX, T *dY)
{
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
    if (nvec < 0) { set_error("nvec < 0"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    T *tmp = nullptr;
    SC_CUDA(cudaMallocAsync(&tmp, sizeof(T) * (size_t)N, c->stream));
    int rc = 0;
    for (int v = 0; v < nvec && !rc; ++v)
        rc = px_vec<T>(c, npc, dX + (i64)v * N, dY + (i64)v * N, tmp, T(1), nullptr, c->stream);
    cudaFreeAsync(tmp, c->stream);
    return rc;
}

}  // namespace sc

using namespace sc;

#define CTX_CHECK(c)                                                              \
    do {                                                                          \
        if (!(c)) { set_error("null context"); return SCALIT_EINVAL; }            \
        if (cudaSetDevice((c)->device) != cudaSuccess) { set_error("cudaSetDevice failed"); return SCALIT_ECUDA; } \
    } while (0)

extern "C" {

const char *scalit_last_error(void) { return g_err; }

void scalit_destroy(scalit_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    double *dptrs[] = {c->H0, c->RES, c->DEP, c->OUTH, c->EIG0, c->VOSB, c->red_partial, c->red_result};
    for (double *p : dptrs) if (p) cudaFree(p);
    float *fptrs[] = {c->H0f, c->RESf, c->DEPf, c->OUTHf, c->EIG0f, c->VOSBf};
    for (float *p : fptrs) if (p) cudaFree(p);
    if (c->VOSBh) cudaFree(c->VOSBh);
    for (int l = 0; l < SCALIT_FMAX; ++l) {
        if (c->tc[l].dig) cudaFree(c->tc[l].dig);
        if (c->tc[l].exps) cudaFree(c->tc[l].exps);
        if (l == 0) { tc_free_px(c); tc32_free(c, true, true); tc16_free(c); }
    }
    if (c->tc_err) cudaFree(c->tc_err);
    if (c->rexp) cudaFree(c->rexp);
    osbw_free(c);
    double *aptrs[] = {c->APP, c->APR, c->AP, c->H0i, c->DEPi, c->OUTHi};
    for (double *p : aptrs) if (p) cudaFree(p);
    for (int i = 0; i < 2; ++i) if (c->qg[i].exec) cudaGraphExecDestroy(c->qg[i].exec);
    if (c->red_counter) cudaFree(c->red_counter);
    if (c->work) cudaFree(c->work);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->cusolver) cusolverDnDestroy((cusolverDnHandle_t)c->cusolver);
    if (c->own_stream) c->stream = c->own_stream;
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->s_in) { cudaStreamSynchronize(c->s_in); cudaStreamDestroy(c->s_in); }
    if (c->s_out) { cudaStreamSynchronize(c->s_out); cudaStreamDestroy(c->s_out); }
    for (int i = 0; i < 6; ++i) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    delete c;
}

int scalit_create(scalit_ctx **out, int nlevel, const int *sizes, const int *dep, int ndvr, int device)
{
    if (!out) { set_error("null output pointer"); return SCALIT_EINVAL; }
    *out = nullptr;
    if (nlevel < 1 || nlevel > SCALIT_FMAX || !sizes) {
        set_error("nlevel=%d out of range 1..%d", nlevel, SCALIT_FMAX);
        return SCALIT_EINVAL;
    }
    scalit_ctx *c = new scalit_ctx();
    Layout &L = c->L;
    L.nlev = nlevel;
    L.ndvr = ndvr ? 1 : 0;
    i64 N = 1;
    for (int i = 0; i < nlevel; ++i) {
        if (sizes[i] < 1 || sizes[i] > 4096) {
            set_error("level %d size %d out of range 1..4096", i + 1, sizes[i]);
            delete c;
            return SCALIT_EINVAL;
        }
        L.n[i] = sizes[i];
        L.dep[i] = (dep && i > 0) ? (dep[i] != 0) : 0;   // sDEP(1) forced false
        N *= sizes[i];
        if (N > 2147483647LL) { set_error("grid of more than 2^31-1 points"); delete c; return SCALIT_EINVAL; }
    }
    if (L.ndvr) L.dep[nlevel - 1] = 0;
    L.compute();
    int rc = ctx_base_init(c, device);
    if (rc) { scalit_destroy(c); return rc; }
    auto alloc2 = [&](double **d, float **f, i64 n) -> int {
        if (n <= 0) return 0;
        SC_CUDA(cudaMalloc(d, sizeof(double) * (size_t)n));
        SC_CUDA(cudaMalloc(f, sizeof(float) * (size_t)n));
        return 0;
    };
    rc = alloc2(&c->H0, &c->H0f, L.h0len);
    if (!rc) rc = alloc2(&c->RES, &c->RESf, L.N);
    if (!rc) rc = alloc2(&c->DEP, &c->DEPf, L.deplen);
    if (!rc) rc = alloc2(&c->OUTH, &c->OUTHf, L.outhlen);
    if (!rc) rc = alloc2(&c->EIG0, &c->EIG0f, L.N);
    if (!rc) rc = alloc2(&c->VOSB, &c->VOSBf, L.vlen);
    if (rc) { scalit_destroy(c); return rc; }
    *out = c;
    return 0;
}

long long scalit_npoints(const scalit_ctx *c) { return c ? c->L.N : -1; }
long long scalit_h0_len(const scalit_ctx *c) { return c ? c->L.h0len : -1; }
long long scalit_dep_len(const scalit_ctx *c) { return c ? c->L.deplen : -1; }
long long scalit_vosb_len(const scalit_ctx *c) { return c ? c->L.vlen : -1; }

int scalit_load(scalit_ctx *c, const double *H0, const double *RES, const double *DEP, const double *OUTH)
{
    CTX_CHECK(c);
    const Layout &L = c->L;
    if (!H0 && L.h0len > 0) { set_error("H0 is required"); return SCALIT_EINVAL; }
    if (!RES) { set_error("RES is required"); return SCALIT_EINVAL; }
    if (L.deplen > 0 && !DEP) { set_error("DEP is required: a level depends on the coordinates"); return SCALIT_EINVAL; }
    if (L.outhlen > 0 && !OUTH) { set_error("OUTH is required when the outer layer is per point"); return SCALIT_EINVAL; }
    c->cxh = false;   // a complex Hamiltonian's imaginary parts apply again only through scalit_load_cx
    if (!all_finite(H0, L.h0len) || !all_finite(RES, L.N) || (L.deplen && !all_finite(DEP, L.deplen)) ||
        (L.outhlen && !all_finite(OUTH, L.outhlen))) {
        set_error("non-finite value in the Hamiltonian input");
        return SCALIT_ENONFINITE;
    }
    cudaStream_t s = c->stream;
    auto up = [&](double *d, float *f, const double *h, i64 n) -> int {
        if (n <= 0) return 0;
        SC_CUDA(cudaMemcpyAsync(d, h, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, s));
        return to_f32(d, f, n, s);
    };
    int rc = up(c->H0, c->H0f, H0, L.h0len);
    if (!rc) rc = up(c->RES, c->RESf, RES, L.N);
    if (!rc) rc = up(c->DEP, c->DEPf, DEP, L.deplen);
    if (!rc) rc = up(c->OUTH, c->OUTHf, OUTH, L.outhlen);
    if (!rc) rc = up(c->EIG0, c->EIG0f, RES, L.N);
    if (rc) return rc;
    SC_CUDA(cudaStreamSynchronize(s));
    rc = tc_prepare(c);
    if (!rc) rc = tc32_prepare(c, false);
    if (!rc) rc = tc16_prepare(c);
    if (!rc) rc = tc64p_prepare(c);
    if (rc) return rc;
    memset(c->tile_pick, -1, sizeof(c->tile_pick));
    rc = gemm_autotune(c, 16);
    if (rc) return rc;
    c->loaded = true;
    c->osb_built = false;
    osbw_invalidate(c);
    c->gen++;
    return 0;
}

int scalit_tile_picks(scalit_ctx *c, int *picks)
{
    CTX_CHECK(c);
    if (!picks) { set_error("null output"); return SCALIT_EINVAL; }
    int k = 0;
    for (int p = 0; p < 2; ++p)
        for (int l = 0; l < c->L.nlev; ++l)
            for (int m = 0; m < 2; ++m) picks[k++] = c->tile_pick[p][l][m];
    return 0;
}

int scalit_set_fp64_mode(scalit_ctx *c, int mode)
{
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (mode != SCALIT_FP64_DFMA && mode != SCALIT_FP64_TENSOR) { set_error("unknown FP64 mode %d", mode); return SCALIT_EINVAL; }
    c->fp64_mode = mode;
    c->gen++;
    return 0;
}

int scalit_set_build_precision(scalit_ctx *c, int precision)
{
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (precision != SCALIT_PREC_FP64 && precision != SCALIT_PREC_FP32) {
        set_error("unknown build precision %d", precision);
        return SCALIT_EINVAL;
    }
    c->build_prec = precision;
    return 0;
}

int scalit_set_fp32_px_storage(scalit_ctx *c, int bits)
{
    CTX_CHECK(c);
    if (bits != 32 && bits != 16) { set_error("FP32 P*X storage of %d bits", bits); return SCALIT_EINVAL; }
    c->px_bits = bits;
    c->gen++;
    return px_half_prepare(c);
}

int scalit_set_fp32_mode(scalit_ctx *c, int mode)
{
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (mode != SCALIT_FP32_SIMT && mode != SCALIT_FP32_TENSOR && mode != SCALIT_FP32_TENSOR_PX &&
        mode != SCALIT_FP32_TENSOR16) {
        set_error("unknown FP32 mode %d", mode);
        return SCALIT_EINVAL;
    }
    c->fp32_mode = mode;
    c->gen++;
    return 0;
}

void *scalit_get_stream(const scalit_ctx *c) { return c ? (void *)c->stream : nullptr; }

int scalit_set_stream(scalit_ctx *c, void *stream)
{
    CTX_CHECK(c);
    SC_CUDA(cudaStreamSynchronize(c->stream));
    if (!c->own_stream) c->own_stream = c->stream;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return 0;
}

int scalit_set_shift(scalit_ctx *c, double e0)
{
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (!std::isfinite(e0)) { set_error("non-finite shift"); return SCALIT_ENONFINITE; }
    c->E0 = e0;
    c->gen++;
    return 0;
}

int scalit_set_precond(scalit_ctx *c, int kind, double de, double beta)
{
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (kind < 1 || kind > 4) { set_error("unknown preconditioner kind %d", kind); return SCALIT_EINVAL; }
    if (kind == SCALIT_TOSBW && !(c->osbw_len > 0 && c->osbw_valid)) {
        set_error("TOSBW needs a window for the current preconditioner: call scalit_build_osbw or scalit_set_osbw");
        return SCALIT_ESTATE;
    }
    if ((kind == SCALIT_TOSBD1 || kind == SCALIT_TOSBD2) && !(fabs(de) > 0.0)) {
        set_error("windowed preconditioner needs DE != 0");
        return SCALIT_EINVAL;
    }
    c->osb_kind = kind;
    c->gen++;
    c->osb_de = fabs(de);
    c->osb_beta = beta;
    return 0;
}

// --------------------------------------------------------------- H * X ---
int scalit_hx_device(scalit_ctx *c, int ntype, int nvec, const double *dX, double *dY)
{
    CTX_CHECK(c);
    return hx_many<double>(c, ntype, nvec, dX, dY);
}

int scalit_hx_level_times(scalit_ctx *c, int precision, int ntype, int nvec, const void *dX, void *dY, int reps,
                          float *ms)
{
    CTX_CHECK(c);
    if (!ms || reps < 1 || nvec < 1 || nvec > 64) { set_error("level timing needs ms, reps >= 1, 1 <= nvec <= 64"); return SCALIT_EINVAL; }
    if (precision != SCALIT_PREC_FP64 && precision != SCALIT_PREC_FP32) { set_error("unknown precision %d", precision); return SCALIT_EINVAL; }
    const int nl = c->L.nlev;
    cudaEvent_t ev[SCALIT_FMAX + 1];
    for (int l = 0; l <= nl; ++l) SC_CUDA(cudaEventCreate(&ev[l]));
    for (int l = 0; l < nl; ++l) ms[l] = 0.0f;
    int rc = 0;
    c->lev_ev = ev;
    for (int r = 0; r < reps && !rc; ++r) {
        rc = precision == SCALIT_PREC_FP64
                 ? hx_many<double>(c, ntype, nvec, static_cast<const double *>(dX), static_cast<double *>(dY))
                 : hx_many<float>(c, ntype, nvec, static_cast<const float *>(dX), static_cast<float *>(dY));
        if (!rc && cudaEventSynchronize(ev[nl]) != cudaSuccess) { set_error("level timing failed"); rc = SCALIT_ECUDA; }
        for (int l = 0; l < nl && !rc; ++l) {
            float t = 0.0f;
            if (cudaEventElapsedTime(&t, ev[l], ev[l + 1]) != cudaSuccess) { set_error("level timing failed"); rc = SCALIT_ECUDA; }
            ms[l] += t / reps;
        }
    }
    c->lev_ev = nullptr;
    for (int l = 0; l <= nl; ++l) cudaEventDestroy(ev[l]);
    return rc;
}

int scalit_level_device(scalit_ctx *c, int level, int accumulate, const double *dX, double *dY)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("level product before scalit_load"); return SCALIT_ESTATE; }
    if (level < 1 || level > c->L.nlev) { set_error("level %d out of range", level); return SCALIT_EINVAL; }
    if (c->fp64_mode == SCALIT_FP64_TENSOR && tc_usable(c, level - 1))
        return tc_level_apply(c, level - 1, dX, dY, accumulate ? 1 : 0, nullptr, 0.0, 1.0, nullptr, c->stream, 1);
    return level_apply<double>(c, level - 1, c->H0, c->DEP, c->OUTH, dX, dY, accumulate ? 1 : 0, nullptr,
                               0.0, 1.0, nullptr, c->stream);
}

int scalit_hx_f32_device(scalit_ctx *c, int ntype, int nvec, const float *dX, float *dY)
{
    CTX_CHECK(c);
    return hx_many<float>(c, ntype, nvec, dX, dY);
}

int scalit_hx(scalit_ctx *c, int ntype, int nvec, const double *X, double *Y)
{
    CTX_CHECK(c);
    if (nvec <= 0) return nvec < 0 ? (set_error("nvec < 0"), SCALIT_EINVAL) : 0;
    if (!c->loaded) { set_error("H*X before scalit_load"); return SCALIT_ESTATE; }
    // Chunks of vectors in two device buffer sets; the copy-in of chunk k+1 and
    // the copy-out of chunk k-1 overlap the product of chunk k (three streams).
    // The chunks grow 1, 2, 4 .. up to G vectors and shrink the same way at the
    // end, so only one vector's copy-in and one vector's copy-out are exposed
    // (a copy of a vector takes about half its product's time) while the
    // middle chunks run the product on several vectors at once.
    const i64 N = c->L.N;
    const i64 target = (256LL << 20) / (8 * N);
    const int G = (int)std::max<i64>(1, std::min<i64>(std::min<i64>(target, 4), nvec));
    std::vector<int> sizes;
    {
        std::vector<int> up;
        for (int g = 1; g < G; g *= 2) up.push_back(g);
        int su = 0;
        for (int g : up) su += g;
        if (2 * su >= nvec) {
            sizes.push_back(1);
            int rem = nvec - 1;
            while (rem > 1) { const int g = std::min(2, rem - 1); sizes.push_back(g); rem -= g; }
            if (rem == 1) sizes.push_back(1);
        } else {
            sizes = up;
            for (int mid = nvec - 2 * su; mid > 0;) { const int g = std::min(G, mid); sizes.push_back(g); mid -= g; }
            for (auto it = up.rbegin(); it != up.rend(); ++it) sizes.push_back(*it);
        }
    }
    double *w = nullptr;
    int rc = work_get(c, sizeof(double) * 4 * (size_t)G * N, (void **)&w);
    if (rc) return rc;
    double *Xd[2] = {w, w + (i64)G * N}, *Yd[2] = {w + 2 * (i64)G * N, w + 3 * (i64)G * N};
    cudaEvent_t *ev = c->ev;   // [in0, in1, comp0, comp1, out0, out1]
    for (int v0 = 0, k = 0; v0 < nvec; v0 += sizes[k], ++k) {
        const int b = k & 1;
        const int nb = sizes[k];
        const size_t bytes = sizeof(double) * (size_t)nb * N;
        SC_CUDA(cudaStreamWaitEvent(c->s_in, ev[2 + b], 0));
        SC_CUDA(cudaMemcpyAsync(Xd[b], X + (i64)v0 * N, bytes, cudaMemcpyHostToDevice, c->s_in));
        SC_CUDA(cudaEventRecord(ev[b], c->s_in));
        SC_CUDA(cudaStreamWaitEvent(c->stream, ev[b], 0));
        SC_CUDA(cudaStreamWaitEvent(c->stream, ev[4 + b], 0));
        rc = hx_many<double>(c, ntype, nb, Xd[b], Yd[b]);
        if (rc) return rc;
        SC_CUDA(cudaEventRecord(ev[2 + b], c->stream));
        SC_CUDA(cudaStreamWaitEvent(c->s_out, ev[2 + b], 0));
        SC_CUDA(cudaMemcpyAsync(Y + (i64)v0 * N, Yd[b], bytes, cudaMemcpyDeviceToHost, c->s_out));
        SC_CUDA(cudaEventRecord(ev[4 + b], c->s_out));
    }
    SC_CUDA(cudaStreamSynchronize(c->s_out));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return tc_check_error(c);
}

// --------------------------------------------------------------- P * X ---
int scalit_px_device(scalit_ctx *c, int npc, int nvec, const double *dX, double *dY)
{
    CTX_CHECK(c);
    return px_many<double>(c, npc, nvec, dX, dY);
}

int scalit_px_f32_device(scalit_ctx *c, int npc, int nvec, const float *dX, float *dY)
{
    CTX_CHECK(c);
    return px_many<float>(c, npc, nvec, dX, dY);
}

int scalit_px(scalit_ctx *c, int npc, int nvec, const double *X, double *Y)
{
    CTX_CHECK(c);
    if (nvec <= 0) return nvec < 0 ? (set_error("nvec < 0"), SCALIT_EINVAL) : 0;
    const i64 N = c->L.N;
    double *w = nullptr;
    int rc = work_get(c, sizeof(double) * 2 * (size_t)N, (void **)&w);
    if (rc) return rc;
    for (int v = 0; v < nvec; ++v) {
        SC_CUDA(cudaMemcpyAsync(w, X + (i64)v * N, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
        rc = px_many<double>(c, npc, 1, w, w + N);
        if (rc) return rc;
        SC_CUDA(cudaMemcpyAsync(Y + (i64)v * N, w + N, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    }
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

// ---------------------------------------------------------- OSB build ---
int scalit_build_osb(scalit_ctx *c, int bjmax, double bjtol, double *stats)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("build before scalit_load"); return SCALIT_ESTATE; }
    if (bjmax < 0 || !(bjtol >= 0.0)) { set_error("bad block-Jacobi parameters"); return SCALIT_EINVAL; }
    return osb_build(c, bjmax, bjtol, stats);
}

int scalit_selftest_wait(scalit_ctx *c, double seconds)
{
    CTX_CHECK(c);
    return wait_selftest(c, seconds);
}

int scalit_build_times(scalit_ctx *c, double *seconds)
{
    CTX_CHECK(c);
    if (!seconds) { set_error("null output"); return SCALIT_EINVAL; }
    for (int l = 0; l < c->L.nlev; ++l) seconds[l] = c->build_s[l];
    return 0;
}

int scalit_get_osb(scalit_ctx *c, double *VOSB, double *EIG0)
{
    CTX_CHECK(c);
    if (!c->osb_built) { set_error("no preconditioner built"); return SCALIT_ESTATE; }
    if (VOSB) SC_CUDA(cudaMemcpyAsync(VOSB, c->VOSB, sizeof(double) * c->L.vlen, cudaMemcpyDeviceToHost, c->stream));
    if (EIG0) SC_CUDA(cudaMemcpyAsync(EIG0, c->EIG0, sizeof(double) * c->L.N, cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

int scalit_set_osb(scalit_ctx *c, const double *VOSB, const double *EIG0)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("set_osb before scalit_load"); return SCALIT_ESTATE; }
    if (!VOSB || !EIG0) { set_error("VOSB and EIG0 are required"); return SCALIT_EINVAL; }
    if (!all_finite(VOSB, c->L.vlen) || !all_finite(EIG0, c->L.N)) { set_error("non-finite preconditioner"); return SCALIT_ENONFINITE; }
    SC_CUDA(cudaMemcpyAsync(c->VOSB, VOSB, sizeof(double) * c->L.vlen, cudaMemcpyHostToDevice, c->stream));
    SC_CUDA(cudaMemcpyAsync(c->EIG0, EIG0, sizeof(double) * c->L.N, cudaMemcpyHostToDevice, c->stream));
    int rc = to_f32(c->VOSB, c->VOSBf, c->L.vlen, c->stream);
    if (!rc) rc = to_f32(c->EIG0, c->EIG0f, c->L.N, c->stream);
    if (rc) return rc;
    SC_CUDA(cudaStreamSynchronize(c->stream));
    c->osb_built = true;
    osbw_invalidate(c);
    c->gen++;
    rc = tc_prepare_px(c);
    if (!rc) rc = tc32_prepare(c, true);
    if (!rc) rc = px_half_prepare(c);
    return rc;
}

// ---------------------------------------------------------- OSBW window ---
int scalit_build_osbw(scalit_ctx *c, double e0, int count, double *de, int npc, int *hwlen)
{
    CTX_CHECK(c);
    return osbw_make(c, e0, count, de, npc, nullptr, hwlen);
}

int scalit_set_osbw(scalit_ctx *c, double e0, int count, double *de, int npc, const double *hw)
{
    CTX_CHECK(c);
    if (!hw) { set_error("HW is required"); return SCALIT_EINVAL; }
    if (count < 1) { set_error("OSBW window size %d < 1", count); return SCALIT_EINVAL; }
    if (!all_finite(hw, (i64)count * count)) { set_error("non-finite HW"); return SCALIT_ENONFINITE; }
    return osbw_make(c, e0, count, de, npc, hw, nullptr);
}

int scalit_get_osbw(scalit_ctx *c, int *hwlen, int *ind, double *hw)
{
    CTX_CHECK(c);
    if (c->osbw_len <= 0) { set_error("no OSBW window"); return SCALIT_ESTATE; }
    const int m = c->osbw_len;
    if (hwlen) *hwlen = m;
    if (ind) SC_CUDA(cudaMemcpyAsync(ind, c->osbw_ind, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost, c->stream));
    if (hw) SC_CUDA(cudaMemcpyAsync(hw, c->osbw_hw, sizeof(double) * (size_t)m * m, cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

// ------------------------------------------------------------------ QMR --
int scalit_qmr_device(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision,
                      const double *dB, double *dX, double *res, int *iters)
{
    CTX_CHECK(c);
    QmrResult r{};
    int rc = qmr_run(c, ntype, qmrmax, qmrtol, precision, dB, dX, &r);
    if (rc) return rc;
    if (res) *res = r.res;
    if (iters) *iters = r.iters;
    return r.code;
}

int scalit_qmr_device_ex(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision,
                         const double *dB, double *dX, int *code, double *res, int *iters)
{
    CTX_CHECK(c);
    if (!code) { set_error("code is required"); return SCALIT_EINVAL; }
    QmrResult r{};
    int rc = qmr_run(c, ntype, qmrmax, qmrtol, precision, dB, dX, &r);
    if (rc) return rc;
    *code = r.code;
    if (res) *res = r.res;
    if (iters) *iters = r.iters;
    return 0;
}

// QMR on host vectors: B in, X in (start, ntype > 0) and out.
static int qmr_host(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision, const double *B,
                    double *X, QmrResult *r)
{
    const i64 N = c->L.N;
    double *bx = nullptr;
    SC_CUDA(cudaMallocAsync(&bx, sizeof(double) * 2 * (size_t)N, c->stream));
    // every failure below falls through to the one free of bx
    int rc = 0;
    cudaError_t e = cudaMemcpyAsync(bx, B, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && ntype > 0)
        e = cudaMemcpyAsync(bx + N, X, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "QMR right-hand side upload", __FILE__, __LINE__);
    if (!rc) rc = qmr_run(c, ntype, qmrmax, qmrtol, precision, bx, bx + N, r);
    if (!rc) {
        e = cudaMemcpyAsync(X, bx + N, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "QMR solution download", __FILE__, __LINE__);
    }
    cudaFreeAsync(bx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int scalit_qmr(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision, const double *B,
               double *X, double *res, int *iters)
{
    CTX_CHECK(c);
    QmrResult r{};
    int rc = qmr_host(c, ntype, qmrmax, qmrtol, precision, B, X, &r);
    if (rc) return rc;
    if (res) *res = r.res;
    if (iters) *iters = r.iters;
    return r.code;
}

int scalit_qmr_ex(scalit_ctx *c, int ntype, int qmrmax, double qmrtol, int precision, const double *B,
                  double *X, int *code, double *res, int *iters)
{
    CTX_CHECK(c);
    if (!code) { set_error("code is required"); return SCALIT_EINVAL; }
    QmrResult r{};
    int rc = qmr_host(c, ntype, qmrmax, qmrtol, precision, B, X, &r);
    if (rc) return rc;
    *code = r.code;
    if (res) *res = r.res;
    if (iters) *iters = r.iters;
    return 0;
}

// ----------------------------------------------------------------- PIST --
void scalit_pist_default_params(scalit_pist_params *p, int m0, double conv_e0, double conv_tol,
                                int conv_start, int conv_step, int conv_max, int conv_gap,
                                int qmr_max, double qmr_tol)
{
    // setPISTConvParam (src/iterate/module/osbw.pistconv.h:303-333)
    memset(p, 0, sizeof(*p));
    p->e0 = conv_e0;
    p->etol = conv_tol;
    p->ntype = 0;
    p->startcnt = (conv_start < m0) ? 2 * m0 : conv_start;
    p->stepcnt = (conv_step < 1) ? 5 : conv_step;
    p->stepeig = (conv_gap < 1) ? 1 : conv_gap;
    p->m_max = (conv_max < p->startcnt) ? p->startcnt + m0 : conv_max;
    p->m = m0;
    p->qmr_ntype = -1;
    p->qmr_max = qmr_max;
    p->qmr_tol = qmr_tol;
    p->precision = SCALIT_PREC_FP64;
    p->verbose = 0;
    p->orth = 1;
}

int scalit_pist(scalit_ctx *c, const scalit_pist_params *p, const double *x0, double *eig, double *res,
                scalit_pist_info *info)
{
    CTX_CHECK(c);
    if (!p || !x0 || !eig || !res) { set_error("null argument"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *dx = nullptr;
    SC_CUDA(cudaMallocAsync(&dx, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    int rc = pist_ctx(c, p, dx, eig, res, info);
    cudaFreeAsync(dx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int scalit_pist_vectors(scalit_ctx *c, const scalit_pist_params *p, const double *x0, double *eig, double *res,
                        scalit_pist_info *info, double *vectors)
{
    CTX_CHECK(c);
    if (!p || !x0 || !eig || !res) { set_error("null argument"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *dx = nullptr;
    SC_CUDA(cudaMallocAsync(&dx, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    int rc = pist_ctx(c, p, dx, eig, res, info, vectors);
    cudaFreeAsync(dx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int scalit_pist_basis(scalit_ctx *c, const scalit_pist_params *p, const double *x0, double *eig, double *res,
                      scalit_pist_info *info, int *cnt, double *ritz, double *hmat, double *vj)
{
    CTX_CHECK(c);
    if (!p || !x0 || !eig || !res) { set_error("null argument"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *dx = nullptr;
    SC_CUDA(cudaMallocAsync(&dx, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    PistBasisOut b;
    b.cnt = cnt; b.ritz = ritz; b.hmat = hmat; b.vj = vj;
    int rc = pist_ctx(c, p, dx, eig, res, info, nullptr, &b);
    cudaFreeAsync(dx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int scalit_pist_residuals(scalit_ctx *c, const scalit_pist_params *p, const double *x0, double *eig, double *res,
                          scalit_pist_info *info, double *resid)
{
    CTX_CHECK(c);
    if (!p || !x0 || !eig || !res || !resid) { set_error("null argument"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *dx = nullptr;
    SC_CUDA(cudaMallocAsync(&dx, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    int rc = pist_ctx(c, p, dx, eig, res, info, nullptr, nullptr, resid);
    cudaFreeAsync(dx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

int scalit_pist_refined(scalit_ctx *c, const scalit_pist_params *p, const double *x0, double *eig, double *res,
                        scalit_pist_info *info, double resid_tol, int max_steps, double *resid, double *vectors,
                        int *steps)
{
    CTX_CHECK(c);
    if (!p || !x0 || !eig || !res || !resid) { set_error("null argument"); return SCALIT_EINVAL; }
    if (!(resid_tol > 0.0) || max_steps < 0) { set_error("refinement needs resid_tol > 0 and max_steps >= 0"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    double *dx = nullptr;
    SC_CUDA(cudaMallocAsync(&dx, sizeof(double) * (size_t)N, c->stream));
    SC_CUDA(cudaMemcpyAsync(dx, x0, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    int rc = pist_ctx(c, p, dx, eig, res, info, vectors, nullptr, resid, resid_tol, max_steps, steps);
    cudaFreeAsync(dx, c->stream);
    cudaStreamSynchronize(c->stream);
    return rc;
}

// ------------------------------------------------ shifts and batches ---
int scalit_qmr_shifts_device(scalit_ctx *c, int nrhs, const double *shifts, int ntype, int qmrmax, double qmrtol,
                             int precision, const double *dB, double *dX, int *codes, double *res)
{
    CTX_CHECK(c);
    return shifted_qmr(c, nrhs, shifts, ntype, qmrmax, qmrtol, precision, dB, dX, codes, res);
}

int scalit_qmr_shifts_batch(scalit_ctx *const *ctxs, int nprob, int nrhs, const double *shifts, int ntype,
                            int qmrmax, double qmrtol, int precision, const double *const *dB, double *const *dX,
                            int *codes, double *res, double *seconds)
{
    if (!ctxs || nprob < 1) { set_error("empty batch"); return SCALIT_EINVAL; }
    CTX_CHECK(ctxs[0]);
    return batch_qmr(ctxs, nprob, nrhs, shifts, ntype, qmrmax, qmrtol, precision, dB, dX, codes, res, seconds);
}

// ------------------------------------------------------ differentiation --
int scalit_hx_adjoint_device(scalit_ctx *c, int ntype, const double *dX, const double *dYbar, double *dXbar,
                             double *dVbar, double *dH0bar)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("adjoint before scalit_load"); return SCALIT_ESTATE; }
    if (!dX || !dYbar) { set_error("null input"); return SCALIT_EINVAL; }
    return hx_adjoint<double>(c, ntype, dX, dYbar, dXbar, dVbar, dH0bar, c->stream);
}

int scalit_hx_adjoint_f32_device(scalit_ctx *c, int ntype, const float *dX, const float *dYbar, float *dXbar,
                                 float *dVbar, float *dH0bar)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("adjoint before scalit_load"); return SCALIT_ESTATE; }
    if (!dX || !dYbar) { set_error("null input"); return SCALIT_EINVAL; }
    return hx_adjoint<float>(c, ntype, dX, dYbar, dXbar, dVbar, dH0bar, c->stream);
}

int scalit_hx_adjoint(scalit_ctx *c, int ntype, const double *X, const double *Ybar, double *Xbar, double *Vbar,
                      double *H0bar)
{
    CTX_CHECK(c);
    if (!c->loaded) { set_error("adjoint before scalit_load"); return SCALIT_ESTATE; }
    if (!X || !Ybar) { set_error("null input"); return SCALIT_EINVAL; }
    const i64 N = c->L.N, nh = std::max<i64>(c->L.h0len, 1);
    double *w = nullptr;
    cudaStream_t s = c->stream;
    SC_CUDA(cudaMallocAsync(&w, sizeof(double) * (size_t)(4 * N + nh), s));
    double *dX = w, *dY = w + N, *dXb = w + 2 * N, *dVb = w + 3 * N, *dHb = w + 4 * N;
    SC_CUDA(cudaMemcpyAsync(dX, X, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    SC_CUDA(cudaMemcpyAsync(dY, Ybar, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    int rc = hx_adjoint<double>(c, ntype, dX, dY, Xbar ? dXb : nullptr, Vbar ? dVb : nullptr,
                                H0bar ? dHb : nullptr, s);
    if (!rc) {
        if (Xbar) SC_CUDA(cudaMemcpyAsync(Xbar, dXb, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
        if (Vbar) SC_CUDA(cudaMemcpyAsync(Vbar, dVb, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
        if (H0bar) SC_CUDA(cudaMemcpyAsync(H0bar, dHb, sizeof(double) * c->L.h0len, cudaMemcpyDeviceToHost, s));
    }
    cudaFreeAsync(w, s);
    SC_CUDA(cudaStreamSynchronize(s));
    return rc;
}

int scalit_hf_gradients(scalit_ctx *c, int m, const double *psi, int np, const double *dvdp, double *grad)
{
    CTX_CHECK(c);
    if (m < 1 || np < 1 || !psi || !dvdp || !grad) { set_error("bad Hellmann-Feynman arguments"); return SCALIT_EINVAL; }
    const i64 N = c->L.N;
    cudaStream_t s = c->stream;
    double *w = nullptr;
    SC_CUDA(cudaMallocAsync(&w, sizeof(double) * (size_t)((i64)(m + np) * N + (i64)m * np), s));
    double *dpsi = w, *ddv = w + (i64)m * N, *dg = w + (i64)(m + np) * N;
    SC_CUDA(cudaMemcpyAsync(dpsi, psi, sizeof(double) * (size_t)m * N, cudaMemcpyHostToDevice, s));
    SC_CUDA(cudaMemcpyAsync(ddv, dvdp, sizeof(double) * (size_t)np * N, cudaMemcpyHostToDevice, s));
    int rc = hf_gradients(c, m, dpsi, np, ddv, dg);
    if (!rc) SC_CUDA(cudaMemcpyAsync(grad, dg, sizeof(double) * (size_t)m * np, cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(w, s);
    SC_CUDA(cudaStreamSynchronize(s));
    return rc;
}

}  // extern "C"

// ======================================================================
// Fortran drop-in layer
// ======================================================================
namespace sc {

static std::mutex g_fmu;
static int g_fdev = 0;
static scalit_ctx *g_fctx = nullptr;      // module state made by scalit_fortran_init_
static scalit_ctx *g_scratch = nullptr;   // stream + scratch for stand-alone routines
static struct { int ntype = -1, qmrmax = 2000; double tol = 1e-4; int precision = SCALIT_PREC_FP64; int orth = 1; } g_fq;

static scalit_ctx *scratch()
{
    if (g_scratch && g_scratch->device == g_fdev) return g_scratch;
    if (g_scratch) { scalit_destroy(g_scratch); g_scratch = nullptr; }
    scalit_ctx *c = new scalit_ctx();
    if (ctx_base_init(c, g_fdev)) { scalit_destroy(c); return nullptr; }
    g_scratch = c;
    return c;
}

// Device buffers for a stand-alone call, freed on scope exit.
struct Scoped {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit Scoped(cudaStream_t st) : s(st) {}
    template <class T> T *get(i64 n)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * (size_t)std::max<i64>(n, 1)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T *)p;
    }
    ~Scoped()
    {
        cudaStreamSynchronize(s);
        for (void *p : ptrs) cudaFree(p);
    }
};

static void report(const char *who, int rc)
{
    if (rc) fprintf(stderr, "scalit_gb300: %s failed: %s\n", who, scalit_last_error());
}

// Y(nin, nout, blk) = per-level contraction; corx may be null; transpose uses H^T.
static int level_host(int nin, int nout, int blk, const double *H, const double *corx, const double *X,
                      double *Y, int transpose)
{
    scalit_ctx *c = scratch();
    if (!c) return SCALIT_ECUDA;
    std::vector<double> Ht;
    if (transpose && nin == 1) {
        // H^T X for single-point blocks: transpose the small matrix on the host
        Ht.resize((size_t)nout * nout);
        for (int i = 0; i < nout; ++i)
            for (int j = 0; j < nout; ++j) Ht[i + (size_t)nout * j] = H[j + (size_t)nout * i];
        H = Ht.data();
        transpose = 0;
    }
    const i64 n = (i64)nin * nout * blk;
    Scoped sb(c->stream);
    double *dH = sb.get<double>((i64)nout * nout), *dX = sb.get<double>(n), *dY = sb.get<double>(n);
    double *dC = corx ? sb.get<double>(nin) : nullptr;
    if (!dH || !dX || !dY || (corx && !dC)) { set_error("device allocation failed"); return SCALIT_ENOMEM; }
    SC_CUDA(cudaMemcpyAsync(dH, H, sizeof(double) * nout * nout, cudaMemcpyHostToDevice, c->stream));
    SC_CUDA(cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    if (corx) SC_CUDA(cudaMemcpyAsync(dC, corx, sizeof(double) * nin, cudaMemcpyHostToDevice, c->stream));
    GemmArgs<double> g{};
    g.K = nout; g.batch = 1; g.alpha = 1.0; g.C = dY;
    if (nin == 1) {
        g.M = nout; g.N = blk; g.Mi = nout; g.s1 = 1; g.s2 = 0;
        g.A = dH;
        g.a_sk = nout;
        g.B = dX; g.b_sk = 1; g.b_sn = nout; g.c_sn = nout;
        if (dC) { set_error("a dependent single-point level is a scaled product"); return SCALIT_EINVAL; }
    } else {
        g.M = nin * blk; g.N = nout; g.Mi = nin; g.s1 = 1; g.s2 = (i64)nin * nout;
        g.A = dX; g.a_sk = nin;
        g.B = dH;
        if (!transpose) { g.b_sk = nout; g.b_sn = 1; } else { g.b_sk = 1; g.b_sn = nout; }
        g.c_sn = nin;
        g.rowscale = dC;
    }
    int rc = launch_gemm<double>(g, c->stream);
    if (rc) return rc;
    SC_CUDA(cudaMemcpyAsync(Y, dY, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

static int vx_host(int nin, int nout, int blk, const double *V, double *X, int transpose)
{
    scalit_ctx *c = scratch();
    if (!c) return SCALIT_ECUDA;
    const i64 n = (i64)nin * nout * blk;
    Scoped sb(c->stream);
    double *dV = sb.get<double>((i64)nout * nout * blk), *dX = sb.get<double>(n), *dY = sb.get<double>(n);
    if (!dV || !dX || !dY) { set_error("device allocation failed"); return SCALIT_ENOMEM; }
    SC_CUDA(cudaMemcpyAsync(dV, V, sizeof(double) * (size_t)nout * nout * blk, cudaMemcpyHostToDevice, c->stream));
    SC_CUDA(cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    int rc = level_rotate<double>(nin, nout, blk, dV, dX, dY, transpose, nullptr, c->stream);
    if (rc) return rc;
    SC_CUDA(cudaMemcpyAsync(X, dY, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    SC_CUDA(cudaStreamSynchronize(c->stream));
    return 0;
}

template <class T>
__global__ void h3x_blk_kernel(int nin, int nout, int blk, const T *Am, const T *X, T *Y)
{
    const i64 total = (i64)nin * nout * blk;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        const i64 a = e % nin;
        const i64 t = e / nin;
        const int i = (int)(t % nout);
        const i64 b = t / nout;
        const T *xb = X + b * (i64)nin * nout;
        T acc = T(0);
        for (int j = 0; j < nout; ++j) acc = fma(Am[a + (i64)nin * (i + (i64)nout * j)], xb[a + (i64)nin * j], acc);
        Y[e] = acc;
    }
}

// Host-callback operators for the generic QMR / PIST drop-ins.
struct HostQmrOps : QmrOps<double> {
    scalit_ctx *c;
    i64 n;
    scalit_fortran_op fhx, fpx;
    std::vector<double> hin, hout;
    const int *state_done;
    int call(scalit_fortran_op f, const double *in, double *out, const int *gate)
    {
        if (gate) {
            int d = 0;
            SC_CUDA(cudaMemcpyAsync(&d, gate, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            SC_CUDA(cudaStreamSynchronize(c->stream));
            if (d) return 0;
        }
        SC_CUDA(cudaMemcpyAsync(hin.data(), in, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        int ni = (int)n, ierr = 0;
        // a trailing IERR argument (MPI callers) is harmless to pass
        reinterpret_cast<void (*)(const int *, const double *, double *, int *)>(f)(&ni, hin.data(), hout.data(), &ierr);
        SC_CUDA(cudaMemcpyAsync(out, hout.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        return 0;
    }
    int hx(const double *in, double *out, const int *gate) override { return call(fhx, in, out, gate); }
    int px(const double *in, double *out, const int *gate) override { return call(fpx, in, out, gate); }
    bool host_side() const override { return true; }
};

struct HostPistOps : PistOps {
    scalit_ctx *c;
    i64 n;
    scalit_fortran_op fh0x;
    scalit_fortran_linsolv flin;
    std::vector<double> hin, hout;
    int h0x(const double *dX, double *dY) override
    {
        SC_CUDA(cudaMemcpyAsync(hin.data(), dX, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        int ni = (int)n, ierr = 0;
        reinterpret_cast<void (*)(const int *, const double *, double *, int *)>(fh0x)(&ni, hin.data(), hout.data(), &ierr);
        SC_CUDA(cudaMemcpyAsync(dY, hout.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        return 0;
    }
    int linsolv(const double *dB, double *dX, int *num) override
    {
        SC_CUDA(cudaMemcpyAsync(hin.data(), dB, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        int ni = (int)n;
        double r = 0.0;
        *num = flin(&ni, hin.data(), hout.data(), &r);
        SC_CUDA(cudaMemcpyAsync(dX, hout.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        SC_CUDA(cudaStreamSynchronize(c->stream));
        return 0;
    }
};

static int qmr_fortran(int ntype, int qmrmax, double tol, int n, const double *B, scalit_fortran_op hx,
                       scalit_fortran_op px, double *X, double *RES, bool mpi_codes)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    *RES = 0.0;
    if (hx == scalit_ehx_ && px == scalit_epx_ && g_fctx && g_fctx->L.N == n) {
        scalit_ctx *f = g_fctx;
        if (cudaSetDevice(f->device) != cudaSuccess) return -10;
        Scoped sb(f->stream);
        double *dB = sb.get<double>(n), *dX = sb.get<double>(n);
        if (!dB || !dX) return -10;
        cudaMemcpyAsync(dB, B, sizeof(double) * n, cudaMemcpyHostToDevice, f->stream);
        if (ntype > 0) cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, f->stream);
        QmrResult r{};
        int rc = qmr_run(f, ntype, qmrmax, tol, g_fq.precision, dB, dX, &r);
        if (rc) { report("qmr (device)", rc); return -10; }
        cudaMemcpyAsync(X, dX, sizeof(double) * n, cudaMemcpyDeviceToHost, f->stream);
        cudaStreamSynchronize(f->stream);
        *RES = r.res;
        int code = r.code;
        if (!mpi_codes && r.breakdown) code = (r.iters > 0) ? -r.iters : 0;
        return code;
    }
    scalit_ctx *c = scratch();
    if (!c) return -10;
    Scoped sb(c->stream);
    double *dB = sb.get<double>(n), *dX = sb.get<double>(n);
    if (!dB || !dX) return -10;
    if (cudaMemcpyAsync(dB, B, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return -10;
    if (ntype > 0 && cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) return -10;
    HostQmrOps ops;
    ops.c = c; ops.n = n; ops.fhx = hx; ops.fpx = px;
    ops.hin.resize(n); ops.hout.resize(n);
    QmrResult r{};
    int rc = qmr_core<double>(c, n, ops, ntype, qmrmax, tol, dB, dX, &r);
    if (rc) { report("qmr", rc); return -10; }
    cudaMemcpyAsync(X, dX, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    *RES = r.res;
    int code = r.code;
    if (!mpi_codes && r.breakdown) code = (r.iters > 0) ? -r.iters : 0;
    return code;
}

static int pist_fortran(double e0, double etol, int ntype, int n, const double *X, int startcnt, int stepcnt,
                        int stepeig, int m, int m_max, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv,
                        double *EIG, double *RES)
{
    scalit_pist_params p{};
    p.e0 = e0; p.etol = etol; p.ntype = ntype; p.startcnt = startcnt; p.stepcnt = stepcnt;
    p.stepeig = stepeig; p.m = m; p.m_max = m_max;
    p.qmr_ntype = g_fq.ntype; p.qmr_max = g_fq.qmrmax; p.qmr_tol = g_fq.tol; p.precision = g_fq.precision;
    p.orth = g_fq.orth;
    const bool own = (h0x == scalit_hx0_ && linsolv == scalit_osb_qmr_ && g_fctx && g_fctx->L.N == n);
    if (own) {
        int rc = scalit_pist(g_fctx, &p, X, EIG, RES, nullptr);
        if (rc < -100) report("pist (device)", rc);
        return rc;
    }
    scalit_ctx *c = scratch();
    if (!c) return 0;
    Scoped sb(c->stream);
    double *dx = sb.get<double>(n);
    if (!dx) return 0;
    cudaMemcpyAsync(dx, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    HostPistOps ops;
    ops.c = c; ops.n = n; ops.fh0x = h0x; ops.flin = linsolv;
    ops.hin.resize(n); ops.hout.resize(n);
    int rc = pist_core(c, n, &p, dx, ops, EIG, RES, nullptr);
    if (rc < -100) report("pist", rc);
    return rc;
}

}  // namespace sc

extern "C" {

void h1x_xyz_(const int *nin, const int *nout, const int *blk, const double *H1, const double *X, double *Y)
{
    report("h1x_xyz", level_host(*nin, *nout, *blk, H1, nullptr, X, Y, 0));
}

void h1x_xyz_seq_(const int *nin, const int *nout, const int *blk, const double *H1, const double *X, double *Y)
{
    report("h1x_xyz_seq", level_host(*nin, *nout, *blk, H1, nullptr, X, Y, 0));
}

void h1tx_xyz_seq_(const int *nin, const int *nout, const int *blk, const double *H1, const double *X, double *Y)
{
    report("h1tx_xyz_seq", level_host(*nin, *nout, *blk, H1, nullptr, X, Y, 1));
}

void h1x_dep_(const int *nin, const int *nout, const int *blk, const double *H1, const double *CORX,
              const double *X, double *Y)
{
    if (*nin == 1) {
        // a one-point dependent factor is a scale of the whole product
        std::vector<double> H(H1, H1 + (size_t)(*nout) * (*nout));
        for (double &h : H) h *= CORX[0];
        report("h1x_dep", level_host(*nin, *nout, *blk, H.data(), nullptr, X, Y, 0));
        return;
    }
    report("h1x_dep", level_host(*nin, *nout, *blk, H1, CORX, X, Y, 0));
}

void h2x_dep_seq_(const int *nin, const int *nout, const int *blk, const double *H1, const double *DEPX,
                  const double *X, double *Y)
{
    h1x_dep_(nin, nout, blk, H1, DEPX, X, Y);
}

void h3x_out_seq_(const int *nin, const int *nout, const int *blk, const double *OUTH, const double *X, double *Y)
{
    scalit_ctx *c = scratch();
    if (!c) return;
    const i64 n = (i64)(*nin) * (*nout) * (*blk);
    const i64 na = (i64)(*nin) * (*nout) * (*nout);
    Scoped sb(c->stream);
    double *dA = sb.get<double>(na), *dX = sb.get<double>(n), *dY = sb.get<double>(n);
    if (!dA || !dX || !dY) { report("h3x_out_seq", SCALIT_ENOMEM); return; }
    cudaMemcpyAsync(dA, OUTH, sizeof(double) * na, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    const int grid = (int)std::min<i64>((n + 255) / 256, 152 * 16);
    h3x_blk_kernel<double><<<std::max(grid, 1), 256, 0, c->stream>>>(*nin, *nout, *blk, dA, dX, dY);
    cudaMemcpyAsync(Y, dY, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { set_error("h3x_out_seq: %s", cudaGetErrorString(e)); report("h3x_out_seq", SCALIT_ECUDA); }
}

void vx_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X)
{
    report("vx", vx_host(*nin, *nout, *blk, VOUT, X, 0));
}

void vtx_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X)
{
    report("vtx", vx_host(*nin, *nout, *blk, VOUT, X, 1));
}

void vx_seq_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X)
{
    vx_(nin, nout, blk, VOUT, X);
}

void vtx_seq_(const int *nin, const int *nout, const int *blk, const double *VOUT, double *X)
{
    vtx_(nin, nout, blk, VOUT, X);
}

static int hosbdiag_host(int bjmax, double bjtol, int blk, int mak, int ndk, double *HOSB, double *VOSB,
                         double *EIG)
{
    scalit_ctx *c = scratch();
    if (!c) return SCALIT_ECUDA;
    const i64 nh = (i64)ndk * mak * mak * blk, nv = (i64)mak * mak * blk, ne = (i64)ndk * mak * blk;
    Scoped sb(c->stream);
    double *dH = sb.get<double>(nh), *dV = sb.get<double>(nv), *dE = sb.get<double>(ne);
    if (!dH || !dV || !dE) { report("hosbdiag", SCALIT_ENOMEM); return SCALIT_ENOMEM; }
    cudaMemcpyAsync(dH, HOSB, sizeof(double) * nh, cudaMemcpyHostToDevice, c->stream);
    double stats[5];
    int rc = hosbdiag_device(c, bjmax, bjtol, blk, mak, ndk, dH, dV, dE, stats, c->stream);
    if (rc) { report("hosbdiag", rc); return rc; }
    cudaMemcpyAsync(HOSB, dH, sizeof(double) * nh, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(VOSB, dV, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(EIG, dE, sizeof(double) * ne, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        set_error("hosbdiag: download failed");
        report("hosbdiag", SCALIT_ECUDA);
        return SCALIT_ECUDA;
    }
    // the reference's summary lines (hosbdiag.f90:67-71)
    printf(" Aver. # of Sweeps:%10.5f.    Aver. OffDiag/Diag:%10.6f\n", stats[4] / blk, stats[2] / stats[4]);
    printf(" Jacobi Effi: Min:%10.5f,   Max:%10.5f,  Mean:%10.5f\n", stats[0], stats[1], stats[2] / blk);
    return 0;
}

void hosbdiag_(const int *bjmax, const double *bjtol, const int *blk, const int *mak, const int *ndk,
               double *HOSB, double *VOSB, double *EIGVAL)
{
    hosbdiag_host(*bjmax, *bjtol, *blk, *mak, *ndk, HOSB, VOSB, EIGVAL);
}

void hosbdiag_seq_(const int *bjmax, const double *bjtol, const int *blk, const int *mak, const int *ndk,
                   double *HOSB, double *VOSB, double *EIGVAL, const int *id)
{
    (void)id;
    hosbdiag_host(*bjmax, *bjtol, *blk, *mak, *ndk, HOSB, VOSB, EIGVAL);
}

// HOSBDIAG_MPI (src/iterate/libiterate_mpi/diagmpi/hosbdiag_mpi.f90:5-96) on
// one rank: the whole NDK stack is local, so it is HosbDiag with IERR = 0.
void hosbdiag_mpi_(const int *comm, const int *bjmax, const double *bjtol, const int *blk, const int *mak,
                   const int *ndk, double *HOSB, double *VOSB, double *RES, int *ierr, const int *id)
{
    (void)comm; (void)id;
    const int rc = hosbdiag_host(*bjmax, *bjtol, *blk, *mak, *ndk, HOSB, VOSB, RES);
    if (ierr) *ierr = rc ? 1 : 0;
}

// MJACOBI (src/iterate/libiterate/diag/jacobi.f90:2-83): one joint rotation of
// the (P, Q) plane of HOUT(NIN, NOUT, NOUT) in place; returns the angle.
double mjacobi_(const int *p, const int *q, const int *nout, const int *nin, double *HOUT)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    const int P = *p, Q = *q, no = *nout, ni = *nin;
    if (P < 1 || Q < 1 || P > no || Q > no || P == Q || ni < 1) {
        set_error("mjacobi: plane (%d, %d) outside 1..%d or nin %d", P, Q, no, ni);
        report("mjacobi", SCALIT_EINVAL);
        return 0.0;
    }
    scalit_ctx *c = scratch();
    if (!c) return 0.0;
    const i64 n = (i64)ni * no * no;
    Scoped sb(c->stream);
    double *dH = sb.get<double>(n), *dabc = sb.get<double>(4);
    if (!dH || !dabc) { report("mjacobi", SCALIT_ENOMEM); return 0.0; }
    double x = 0.0;
    int rc = cudaMemcpyAsync(dH, HOUT, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, c->stream) == cudaSuccess
                 ? 0 : SCALIT_ECUDA;
    if (!rc) rc = mjacobi_device(P, Q, no, ni, dH, dabc, &x, c->stream);
    if (!rc && (cudaMemcpyAsync(HOUT, dH, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess))
        rc = SCALIT_ECUDA;
    if (rc) { report("mjacobi", rc); return 0.0; }
    return x;
}

static double dot_host(int n, const double *X, const double *Y, int *ierr)
{
    if (ierr) *ierr = 0;
    scalit_ctx *c = scratch();
    if (!c || n <= 0) { if (ierr && n > 0) *ierr = 1; return 0.0; }
    Scoped sb(c->stream);
    double *dX = sb.get<double>(n), *dY = (Y == X) ? dX : sb.get<double>(n), *dr = sb.get<double>(1);
    if (!dX || !dY || !dr) { if (ierr) *ierr = 1; return 0.0; }
    cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    if (Y != X) cudaMemcpyAsync(dY, Y, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    double r = 0.0;
    if (dot_dev<double>(c, n, dX, dY, dr, c->stream) || sync_read_doubles(c, dr, &r, 1)) {
        if (ierr) *ierr = 1;
        return 0.0;
    }
    return r;
}

double norm_mpi_(const int *comm, const int *nin, const double *X, int *ierr)
{
    (void)comm;
    return sqrt(dot_host(*nin, X, X, ierr));
}

double dotprod_mpi_(const int *comm, const int *nin, const double *X, const double *Y, int *ierr)
{
    (void)comm;
    return dot_host(*nin, X, Y, ierr);
}

static int mgs_host(int n, const double *WJ, int m, double *VJ)
{
    // One-step modified Gram-Schmidt of WJ against VJ(:, 1:m) into VJ(:, m+1).
    scalit_ctx *c = scratch();
    if (!c) return 0;
    Scoped sb(c->stream);
    const i64 total = (i64)n * (m + 1);
    double *dV = sb.get<double>(total), *dd = sb.get<double>(m + 2);
    if (!dV || !dd) return 0;
    if (m > 0) cudaMemcpyAsync(dV, VJ, sizeof(double) * (size_t)n * m, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dV + (i64)n * m, WJ, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    double *v = dV + (i64)n * m;
    double nrm2 = 0.0;
    if (dot_dev<double>(c, n, v, v, dd + m, c->stream) || sync_read_doubles(c, dd + m, &nrm2, 1)) return 0;
    if (nrm2 == 0.0) return 0;
    // Projections one vector at a time in the reference's order.
    for (int i = 0; i < m; ++i) {
        const double *u = dV + (i64)n * i;
        double d = 0.0;
        if (dot_dev<double>(c, n, v, u, dd + i, c->stream) || sync_read_doubles(c, dd + i, &d, 1)) return 0;
        if (axpy_dev(n, -d, u, v, c->stream)) return 0;   // v -= d u
    }
    double nv = 0.0;
    if (dot_dev<double>(c, n, v, v, dd + m + 1, c->stream) || sync_read_doubles(c, dd + m + 1, &nv, 1)) return 0;
    if (nv == 0.0) return 0;
    if (scal_dev(n, 1.0 / sqrt(nv), v, c->stream)) return 0;
    cudaMemcpyAsync(VJ + (i64)n * m, v, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    return 1;
}

int mgs_orth_(const int *n, const double *WJ, const int *m, double *VJ)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    return mgs_host(*n, WJ, *m, VJ);
}

int mgs_orth_mpi_(const int *n, const double *WJ, const int *m, double *VJ, int *ierr)
{
    if (ierr) *ierr = 0;
    std::lock_guard<std::mutex> lk(g_fmu);
    return mgs_host(*n, WJ, *m, VJ);
}

int qmr_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n, const double *B,
         scalit_fortran_op hx, scalit_fortran_op px, double *X, double *RES)
{
    return qmr_fortran(*ntype, *qmrmax, *qmrtol, *n, B, hx, px, X, RES, false);
}

int qmr_mpi_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n, const double *B,
             scalit_fortran_op hx, scalit_fortran_op px, double *X, double *RES, const int *myid)
{
    (void)myid;
    return qmr_fortran(*ntype, *qmrmax, *qmrtol, *n, B, hx, px, X, RES, true);
}

// QMR_CX (src/iterate/libiterate/qmr/qmrcx.f90:4-175) and PIST_CONV_SX
// (src/iterate/libiterate/pist/pist_sx.f90:4-96), the complex library's
// externals, with the caller's callbacks on COMPLEX*16 arrays.
int qmr_cx_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *n, const double *B,
            scalit_fortran_op hx, scalit_fortran_op px, double *X, double *RES)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    *RES = 0.0;
    scalit_ctx *c = scratch();
    if (!c) return -10;
    int code = 0;
    double res = 0.0;
    const int rc = qmr_cx_host(c, *n, hx, px, *ntype, *qmrmax, *qmrtol, B, X, &code, &res);
    if (rc) { report("qmr_cx", rc); return -10; }
    *RES = res;
    return code;
}

static int pist_complex_fortran(const double *e0, const double *etol, const int *ntype, const int *n,
                                const double *X, const int *startcnt, const int *stepcnt, const int *stepeig,
                                const int *m, const int *m_max, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv,
                                double *EIG, double *RES, int conj)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    *RES = 0.0;
    if (*ntype > 0) {
        fprintf(stderr, "scalit_gb300: complex PIST with ntype > 0 has no defined result in the reference\n");
        return 0;
    }
    scalit_ctx *c = scratch();
    if (!c) return 0;
    int status = 0;
    double res = 0.0;
    const int rc = pist_sx_host(c, *n, *e0, *etol, X, *startcnt, *stepcnt, *stepeig, *m, *m_max, h0x, linsolv, EIG,
                                &res, &status, conj);
    if (rc) { report(conj ? "pist_conv_cx" : "pist_conv_sx", rc); return rc; }
    *RES = res;
    return status;
}

int pist_conv_sx_(const double *e0, const double *etol, const int *ntype, const int *n, const double *X,
                  const int *startcnt, const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
                  scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG, double *RES)
{
    return pist_complex_fortran(e0, etol, ntype, n, X, startcnt, stepcnt, stepeig, m, m_max, h0x, linsolv, EIG, RES, 0);
}

// PIST_CONV_CX (src/iterate/libiterate/pist/pist_cx.f90): the conjugate-product twin.
int pist_conv_cx_(const double *e0, const double *etol, const int *ntype, const int *n, const double *X,
                  const int *startcnt, const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
                  scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG, double *RES)
{
    return pist_complex_fortran(e0, etol, ntype, n, X, startcnt, stepcnt, stepeig, m, m_max, h0x, linsolv, EIG, RES, 1);
}

// pistH0 (src/iterate/libiterate/pist/pistHij.f90:70-125) and pistH0_MPI
// (src/iterate/libiterate_mpi/pist/pistHij_mpi.f90:83-190): one block of
// Krylov vectors m_low..m_high and their HMAT columns, with the caller's
// callbacks, on the caller's VJ(N, M_HIGH) and HMAT(M_MAX, M_HIGH).
static int pisth0_fortran(int n, const double *X, int m_max, int m_low, int m_high, scalit_fortran_op h0x,
                          scalit_fortran_linsolv linsolv, double *VJ, double *HMAT, bool mpi, int *num2)
{
    // no lock held here: the callbacks may be this library's own externals
    if (num2) *num2 = 0;
    if (m_low < 1 || m_low >= m_high || m_high > m_max || n < 1) return 0;
    const bool own = (h0x == scalit_hx0_ && linsolv == scalit_osb_qmr_ && g_fctx && g_fctx->L.N == n);
    scalit_ctx *c = own ? g_fctx : scratch();
    if (!c) return 0;
    if (cudaSetDevice(c->device) != cudaSuccess) return 0;
    int ret = 0, rc = 0;
    if (own) {
        // the module's own operators stay on the device: HX0 = MYHX(TA0), LinSolv = OSB_QMR
        struct OwnOps : PistOps {
            scalit_ctx *c;
            int h0x(const double *dX, double *dY) override { return scalit_hx_device(c, SCALIT_TA0, 1, dX, dY); }
            int linsolv(const double *dB, double *dX, int *num) override
            {
                double res = 0.0;
                int it = 0, code = 0;
                const int r = scalit_qmr_device_ex(c, g_fq.ntype, g_fq.qmrmax, g_fq.tol, g_fq.precision, dB, dX,
                                                   &code, &res, &it);
                if (r) return r;
                *num = code;
                return 0;
            }
        } ops;
        ops.c = c;
        rc = pisth0_host(c, n, X, m_max, m_low, m_high, ops, VJ, HMAT, mpi, num2, &ret);
    } else {
        HostPistOps ops;
        ops.c = c; ops.n = n; ops.fh0x = h0x; ops.flin = linsolv;
        ops.hin.resize(n); ops.hout.resize(n);
        rc = pisth0_host(c, n, X, m_max, m_low, m_high, ops, VJ, HMAT, mpi, num2, &ret);
    }
    if (rc) { report(mpi ? "pisth0_mpi" : "pisth0", rc); return 0; }
    return ret;
}

int pisth0_(const int *n, const double *X, const int *m_max, const int *m_low, const int *m_high,
            scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *VJ, double *HMAT)
{
    return pisth0_fortran(*n, X, *m_max, *m_low, *m_high, h0x, linsolv, VJ, HMAT, false, nullptr);
}

int pisth0_mpi_(const int *myid, const int *rootid, const int *n, const double *X, const int *m_max,
                const int *m_low, const int *m_high, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv,
                double *VJ, double *HMAT, int *num2)
{
    (void)myid; (void)rootid;
    return pisth0_fortran(*n, X, *m_max, *m_low, *m_high, h0x, linsolv, VJ, HMAT, true, num2);
}

int pist_conv_(const double *e0, const double *etol, const int *ntype, const int *n, const double *X,
               const int *startcnt, const int *stepcnt, const int *stepeig, const int *m, const int *m_max,
               scalit_fortran_op h0x, scalit_fortran_linsolv linsolv, double *EIG, double *RES)
{
    return pist_fortran(*e0, *etol, *ntype, *n, X, *startcnt, *stepcnt, *stepeig, *m, *m_max, h0x, linsolv,
                        EIG, RES);
}

int pist_conv_mpi_(const int *myid, const int *rootid, const double *e0, const double *etol, const int *ntype,
                   const int *n, const double *X, const int *startcnt, const int *stepcnt, const int *stepeig,
                   const int *m, const int *m_max, scalit_fortran_op h0x, scalit_fortran_linsolv linsolv,
                   double *EIG, double *RES)
{
    (void)myid; (void)rootid;
    return pist_fortran(*e0, *etol, *ntype, *n, X, *startcnt, *stepcnt, *stepeig, *m, *m_max, h0x, linsolv,
                        EIG, RES);
}

void scalit_fortran_device_(const int *device)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    g_fdev = *device;
}

void scalit_fortran_init_(const int *sf, const int *sn, const int *sdep, const double *H0, const double *RES,
                          const double *DEP, const double *e0, int *ierr)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    if (g_fctx) { scalit_destroy(g_fctx); g_fctx = nullptr; }
    int dep[SCALIT_FMAX] = {};
    for (int i = 0; i < *sf && i < SCALIT_FMAX; ++i) dep[i] = sdep[i] != 0;
    int rc = scalit_create(&g_fctx, *sf, sn, dep, 0, g_fdev);
    if (!rc) rc = scalit_load(g_fctx, H0, RES, DEP, nullptr);
    if (!rc) rc = scalit_set_shift(g_fctx, *e0);
    if (rc) { report("scalit_fortran_init", rc); if (g_fctx) { scalit_destroy(g_fctx); g_fctx = nullptr; } }
    if (ierr) *ierr = rc;
}

void scalit_fortran_precond_(const int *sosb, const double *de, const double *beta, const int *bjmax,
                             const double *bjtol, int *ierr)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    // sOSB = TOSBW: the drivers call initOSBW after progDiag (osb.progPX.h:28-35),
    // here scalit_fortran_osbw_, which selects TOSBW once the window exists.
    const int kind = (*sosb == SCALIT_TOSBW) ? SCALIT_TOSB : *sosb;
    int rc = g_fctx ? scalit_set_precond(g_fctx, kind, *de, *beta) : SCALIT_ESTATE;
    if (!rc) rc = scalit_build_osb(g_fctx, *bjmax, *bjtol, nullptr);
    if (rc) report("scalit_fortran_precond", rc);
    if (ierr) *ierr = rc;
}

void scalit_fortran_osbw_(const double *e0, const int *cnt, double *de, const int *npc, int *ierr)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    const int rc = g_fctx ? scalit_build_osbw(g_fctx, *e0, *cnt, de, *npc, nullptr) : SCALIT_ESTATE;
    if (rc) report("scalit_fortran_osbw", rc);
    if (ierr) *ierr = rc;
}

void scalit_fortran_qmr_param_(const int *ntype, const int *qmrmax, const double *qmrtol, const int *precision)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    g_fq.ntype = *ntype;
    g_fq.qmrmax = *qmrmax;
    g_fq.tol = *qmrtol;
    g_fq.precision = *precision;
}

void scalit_fortran_final_(void)
{
    std::lock_guard<std::mutex> lk(g_fmu);
    if (g_fctx) { scalit_destroy(g_fctx); g_fctx = nullptr; }
    if (g_scratch) { scalit_destroy(g_scratch); g_scratch = nullptr; }
}

void scalit_hx0_(const int *n, const double *X, double *Y)
{
    if (!g_fctx || g_fctx->L.N != *n) { fprintf(stderr, "scalit_gb300: scalit_hx0 without a matching scalit_fortran_init\n"); return; }
    report("scalit_hx0", scalit_hx(g_fctx, SCALIT_TA0, 1, X, Y));
}

void scalit_ehx_(const int *n, const double *X, double *Y)
{
    if (!g_fctx || g_fctx->L.N != *n) { fprintf(stderr, "scalit_gb300: scalit_ehx without a matching scalit_fortran_init\n"); return; }
    report("scalit_ehx", scalit_hx(g_fctx, SCALIT_TA1, 1, X, Y));
}

void scalit_epx_(const int *n, const double *X, double *Y)
{
    if (!g_fctx || g_fctx->L.N != *n) { fprintf(stderr, "scalit_gb300: scalit_epx without a matching scalit_fortran_init\n"); return; }
    report("scalit_epx", scalit_px(g_fctx, SCALIT_TA1, 1, X, Y));
}

int scalit_osb_qmr_(const int *n, const double *B, double *X, double *ERES)
{
    if (!g_fctx || g_fctx->L.N != *n) { fprintf(stderr, "scalit_gb300: scalit_osb_qmr without a matching scalit_fortran_init\n"); return -10; }
    int iters = 0;
    int code = scalit_qmr(g_fctx, g_fq.ntype, g_fq.qmrmax, g_fq.tol, g_fq.precision, B, X, ERES, &iters);
    if (code < -100) { report("scalit_osb_qmr", code); return -10; }
    return code;
}

}  // extern "C"
