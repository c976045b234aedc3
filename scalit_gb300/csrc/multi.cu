// Shifted systems and batches of problems: QMR on nrhs right-hand sides at
// once, right-hand side v solving (H - E_v) x_v = b_v with the preconditioner's
// kernel shifted to E_v as well, and many independent problems advanced
// together by one CUDA graph with a branch per problem.
//
// The reference solves one system per QMR call (qmr.f90:5-175, called by
// OSB_QMR once per Krylov step); solving several shifts of one Hamiltonian and
// many small problems per launch is this library's extension for workloads
// that would otherwise leave most of the GPU idle.
#include "internal.cuh"

#include <algorithm>
#include <vector>

namespace sc {

// The context's operators on nrhs vectors with per-vector shifts.
template <class T> struct CtxMultiOps : QmrOps<T> {
    scalit_ctx *c = nullptr;
    int nrhs = 1;
    const T *shiftv = nullptr;     // device, nrhs
    const double *e0v = nullptr;   // device, nrhs
    const int *vgate = nullptr;    // the right-hand sides' stop flags (set after setup)
    int vstride = 0;
    T *tmp = nullptr;
    void set_scratch(T *p) override { tmp = p; }
    int hx(const T *in, T *out, const int *gate) override
    {
        return hx_batch<T>(c, in, out, nrhs, T(0), T(1), gate, c->stream, shiftv, vgate, vstride);
    }
    int px(const T *in, T *out, const int *gate) override
    {
        return px_multi<T>(c, in, out, tmp, nrhs, e0v, gate, c->stream, vgate, vstride);
    }
};

__global__ void shifts_to_f32_kernel(int n, const double *x, float *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

// Per-problem resources of a shifted solve: the shift arrays and, in FP32, the
// converted right-hand sides and solutions.
struct ShiftedJob {
    scalit_ctx *c = nullptr;
    int nrhs = 0, precision = SCALIT_PREC_FP64;
    double *e0v = nullptr;     // device, nrhs (FP64 shifts, also FP64 H*X shifts)
    float *shiftf = nullptr;   // device, nrhs (FP32 H*X shifts)
    float *bx = nullptr;       // FP32: B then X, n x nrhs each
    CtxMultiOps<double> ops64;
    CtxMultiOps<float> ops32;
    QmrSolve<double> q64;
    QmrSolve<float> q32;

    int begin(scalit_ctx *ctx, int nr, const double *shifts, int prec, int ntype, int qmrmax, double tol,
              const double *dB, const double *dX)
    {
        c = ctx; nrhs = nr; precision = prec;
        if (!c->osb_built) { set_error("QMR needs the preconditioner: build or load it first"); return SCALIT_ESTATE; }
        if (prec != SCALIT_PREC_FP64 && prec != SCALIT_PREC_FP32) { set_error("unknown precision %d", prec); return SCALIT_EINVAL; }
        const i64 n = c->L.N, nn = n * nrhs;
        cudaStream_t s = c->stream;
        SC_CUDA(cudaMallocAsync(&e0v, sizeof(double) * nrhs, s));
        SC_CUDA(cudaMemcpyAsync(e0v, shifts, sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
        SC_CUDA(cudaStreamSynchronize(s));   // the host shifts may go away after return
        if (prec == SCALIT_PREC_FP64) {
            ops64.c = c; ops64.nrhs = nrhs; ops64.shiftv = e0v; ops64.e0v = e0v;
            int r = q64.setup(c, n, nrhs, &ops64, ntype, qmrmax, tol, dB, dX, s);
            // a right-hand side that stopped costs no more operator work
            ops64.vgate = qmr_done_flag(q64.st);
            ops64.vstride = qmr_state_stride();
            return r;
        }
        SC_CUDA(cudaMallocAsync(&shiftf, sizeof(float) * nrhs, s));
        shifts_to_f32_kernel<<<(nrhs + 127) / 128, 128, 0, s>>>(nrhs, e0v, shiftf);
        SC_CHECK_LAUNCH();
        SC_CUDA(cudaMallocAsync(&bx, sizeof(float) * 2 * (size_t)nn, s));
        int rc = to_f32(dB, bx, nn, s);
        if (!rc && ntype > 0) rc = to_f32(dX, bx + nn, nn, s);
        if (rc) return rc;
        ops32.c = c; ops32.nrhs = nrhs; ops32.shiftv = shiftf; ops32.e0v = e0v;
        rc = q32.setup(c, n, nrhs, &ops32, ntype, qmrmax, tol, bx, bx + nn, s);
        ops32.vgate = qmr_done_flag(q32.st);
        ops32.vstride = qmr_state_stride();
        return rc;
    }
    int iteration() { return precision == SCALIT_PREC_FP64 ? q64.iteration() : q32.iteration(); }
    const int *gate() const { return precision == SCALIT_PREC_FP64 ? q64.gate : q32.gate; }
    int end(double *dX, QmrResult *out)
    {
        const i64 nn = c->L.N * nrhs;
        int rc;
        if (precision == SCALIT_PREC_FP64) {
            rc = q64.finish(dX, out);
        } else {
            rc = q32.finish(bx + nn, out);
            if (!rc) rc = to_f64(bx + nn, dX, nn, c->stream);
        }
        release();
        return rc;
    }
    void release()
    {
        cudaStream_t s = c ? c->stream : nullptr;
        if (e0v) cudaFreeAsync(e0v, s);
        if (shiftf) cudaFreeAsync(shiftf, s);
        if (bx) cudaFreeAsync(bx, s);
        if (s) cudaStreamSynchronize(s);
        e0v = nullptr; shiftf = nullptr; bx = nullptr;
    }
};

static void store_results(const std::vector<QmrResult> &r, int *codes, double *res, size_t off)
{
    for (size_t v = 0; v < r.size(); ++v) {
        if (codes) codes[off + v] = r[v].code;
        if (res) res[off + v] = r[v].res;
    }
}

int shifted_qmr(scalit_ctx *c, int nrhs, const double *shifts, int ntype, int qmrmax, double tol, int precision,
                const double *dB, double *dX, int *codes, double *res)
{
    if (nrhs < 1 || nrhs > 65535) { set_error("nrhs must be in 1..65535"); return SCALIT_EINVAL; }
    if (!shifts || !dB || !dX) { set_error("null argument"); return SCALIT_EINVAL; }
    // one problem: the solver's own loop (graph captured per call)
    ShiftedJob job;
    int rc = job.begin(c, nrhs, shifts, precision, ntype, qmrmax, tol, dB, dX);
    if (rc) { job.release(); return rc; }
    const int batch = 4;
    cudaStream_t s = c->stream;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int b = 0; b < batch && !rc; ++b) rc = job.iteration();
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (!rc && ce != cudaSuccess) rc = cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    if (!rc && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "cudaGraphInstantiate", __FILE__, __LINE__);
    if (graph) cudaGraphDestroy(graph);
    int *h_flag = reinterpret_cast<int *>(c->h_pinned);
    for (int it = 0; !rc; it += batch) {
        if (cudaGraphLaunch(exec, s) != cudaSuccess ||
            cudaMemcpyAsync(h_flag, job.gate(), sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "shifted QMR", __FILE__, __LINE__); break; }
        if (*h_flag) break;
        if (it > qmrmax + batch) { set_error("QMR did not stop"); rc = SCALIT_ESTATE; }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (rc) { job.release(); return rc; }
    std::vector<QmrResult> out((size_t)nrhs);
    rc = job.end(dX, out.data());
    if (!rc) store_results(out, codes, res, 0);
    return rc;
}

int batch_qmr(scalit_ctx *const *ctxs, int nprob, int nrhs, const double *shifts, int ntype, int qmrmax,
              double tol, int precision, const double *const *dB, double *const *dX, int *codes, double *res,
              double *seconds)
{
    if (nprob < 1 || !ctxs || !shifts || !dB || !dX) { set_error("null argument or empty batch"); return SCALIT_EINVAL; }
    if (nrhs < 1 || nrhs > 65535) { set_error("nrhs must be in 1..65535"); return SCALIT_EINVAL; }
    for (int p = 0; p < nprob; ++p) {
        if (!ctxs[p]) { set_error("null context %d", p); return SCALIT_EINVAL; }
        if (ctxs[p]->device != ctxs[0]->device) { set_error("a batch runs on one device"); return SCALIT_EINVAL; }
        for (int q = 0; q < p; ++q)
            if (ctxs[q] == ctxs[p] || ctxs[q]->stream == ctxs[p]->stream) { set_error("contexts of a batch need their own streams"); return SCALIT_EINVAL; }
    }
    std::vector<ShiftedJob> jobs((size_t)nprob);
    int rc = 0;
    for (int p = 0; p < nprob && !rc; ++p)
        rc = jobs[p].begin(ctxs[p], nrhs, shifts + (size_t)p * nrhs, precision, ntype, qmrmax, tol, dB[p], dX[p]);
    for (int p = 0; p < nprob && !rc; ++p)
        if (cudaStreamSynchronize(ctxs[p]->stream) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "batch setup", __FILE__, __LINE__);
    if (rc) { for (auto &j : jobs) if (j.c) j.release(); return rc; }

    // one graph: fork from the first problem's stream, every problem's
    // iterations on its own stream, join back
    const int batch = 4;
    cudaStream_t root = ctxs[0]->stream;
    std::vector<cudaEvent_t> ev((size_t)nprob + 1, nullptr);
    for (auto &e : ev) if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = SCALIT_ECUDA;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (!rc && cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "cudaStreamBeginCapture", __FILE__, __LINE__);
    if (!rc) {
        cudaEventRecord(ev[nprob], root);
        for (int p = 0; p < nprob && !rc; ++p) {
            cudaStream_t sp = ctxs[p]->stream;
            if (sp != root) cudaStreamWaitEvent(sp, ev[nprob], 0);
            for (int b = 0; b < batch && !rc; ++b) rc = jobs[p].iteration();
            if (sp != root) { cudaEventRecord(ev[p], sp); cudaStreamWaitEvent(root, ev[p], 0); }
        }
        const cudaError_t ce = cudaStreamEndCapture(root, &graph);
        if (!rc && ce != cudaSuccess) rc = cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    }
    if (!rc && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "cudaGraphInstantiate", __FILE__, __LINE__);
    if (graph) cudaGraphDestroy(graph);

    // replay until every problem's right-hand sides have stopped
    int *flags = nullptr;
    if (!rc && cudaMallocHost(&flags, sizeof(int) * (size_t)nprob) != cudaSuccess) rc = SCALIT_ENOMEM;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (!rc) { cudaEventCreate(&t0); cudaEventCreate(&t1); cudaEventRecord(t0, root); }
    for (int it = 0; !rc; it += batch) {
        if (cudaGraphLaunch(exec, root) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "cudaGraphLaunch", __FILE__, __LINE__); break; }
        for (int p = 0; p < nprob; ++p)
            cudaMemcpyAsync(flags + p, jobs[p].gate(), sizeof(int), cudaMemcpyDeviceToHost, root);
        if (cudaStreamSynchronize(root) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "batch poll", __FILE__, __LINE__); break; }
        bool all = true;
        for (int p = 0; p < nprob; ++p) all = all && flags[p];
        if (all) break;
        if (it > qmrmax + batch) { set_error("QMR did not stop"); rc = SCALIT_ESTATE; }
    }
    if (!rc && t0) {
        cudaEventRecord(t1, root);
        cudaEventSynchronize(t1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t0, t1);
        if (seconds) *seconds = ms / 1e3;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (flags) cudaFreeHost(flags);
    if (exec) cudaGraphExecDestroy(exec);
    for (auto &e : ev) if (e) cudaEventDestroy(e);
    for (int p = 0; p < nprob; ++p) {
        std::vector<QmrResult> out((size_t)nrhs);
        if (rc) { if (jobs[p].c) jobs[p].release(); continue; }
        int r2 = jobs[p].end(dX[p], out.data());
        if (r2 && !rc) rc = r2;
        if (!r2) store_results(out, codes, res, (size_t)p * nrhs);
    }
    return rc;
}

}  // namespace sc
