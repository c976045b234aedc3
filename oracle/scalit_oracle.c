/*
 * CPU oracle for the ScalIT iterate hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference's serial iterate library
 * (Fortran 90): the H*X product, the OSB preconditioner P*X, the layered
 * block-Jacobi build of the preconditioner, and QMR.  Loop order and
 * summation order follow the cited reference lines so results match the
 * reference's arithmetic term by term.  Only tests, the package's smoke check
 * and the benchmark's CPU-baseline leg may load this library; the product path
 * never does.
 *
 * Parity status: the reference cannot be compiled here (Fortran + MPI, no
 * Fortran compiler) and ships no golden vectors for this path, so this
 * restatement is pinned against the reference's own known-answer test
 * patterns (QMR recovers x0(i)=i: src/iterate/libiterate/qmr/testing/qmr.drv.f90;
 * PIST eigenvalues equal DSYEV's: src/iterate/libiterate/pist/testing/pist.drv.f90)
 * and against independent mathematics (dense Kronecker-sum Hamiltonians,
 * exact inverses), not against outputs of the reference itself.
 *
 * OpenMP parallelises only over independent blocks / independent grid
 * points; every reduction keeps the reference's sequential order, so results
 * do not depend on the thread count.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

typedef long long i64;

#define ORC_FMAX 20

/* ---------------------------------------------------------------------------
 * Per-level contractions.
 * ------------------------------------------------------------------------- */

/* H1X (src/libutil/serial/base/matrix.f90:91-107) applied per block as
 * H1X_XYZ (src/iterate/libiterate/hpx/hpx.f90:5-18):
 *   Y(:,i,b) = H(i,1) X(:,1,b) + sum_{j=2..nout} H(i,j) X(:,j,b). */
void orc_h1x_xyz(int nin, int nout, int blk, const double *H, const double *X, double *Y)
{
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b) {
        const double *Xb = X + (i64)b * nin * nout;
        double *Yb = Y + (i64)b * nin * nout;
        for (int i = 0; i < nout; ++i) {
            double *yo = Yb + (i64)i * nin;
            const double h = H[i];
            for (int a = 0; a < nin; ++a) yo[a] = h * Xb[a];
            for (int j = 1; j < nout; ++j) {
                const double hij = H[i + (i64)j * nout];
                const double *xj = Xb + (i64)j * nin;
                for (int a = 0; a < nin; ++a) yo[a] = yo[a] + hij * xj[a];
            }
        }
    }
}

/* H1TX (matrix.f90:116-130): the transpose, Y(:,i,b) = sum_j H(j,i) X(:,j,b). */
void orc_h1tx_xyz(int nin, int nout, int blk, const double *H, const double *X, double *Y)
{
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b) {
        const double *Xb = X + (i64)b * nin * nout;
        double *Yb = Y + (i64)b * nin * nout;
        for (int i = 0; i < nout; ++i) {
            double *yo = Yb + (i64)i * nin;
            const double h = H[(i64)i * nout];
            for (int a = 0; a < nin; ++a) yo[a] = h * Xb[a];
            for (int j = 1; j < nout; ++j) {
                const double hji = H[j + (i64)i * nout];
                const double *xj = Xb + (i64)j * nin;
                for (int a = 0; a < nin; ++a) yo[a] = yo[a] + hji * xj[a];
            }
        }
    }
}

/* H2X (matrix.f90:139-155) per block as H1X_DEP (hpx.f90:21-35):
 *   Y(:,i,b) = sum_j (H(i,j) * CORX(:)) * X(:,j,b)   (Fortran evaluates a*b*c as (a*b)*c). */
void orc_h1x_dep(int nin, int nout, int blk, const double *H, const double *corx,
                 const double *X, double *Y)
{
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b) {
        const double *Xb = X + (i64)b * nin * nout;
        double *Yb = Y + (i64)b * nin * nout;
        for (int i = 0; i < nout; ++i) {
            double *yo = Yb + (i64)i * nin;
            const double h = H[i];
            for (int a = 0; a < nin; ++a) yo[a] = (h * corx[a]) * Xb[a];
            for (int j = 1; j < nout; ++j) {
                const double hij = H[i + (i64)j * nout];
                const double *xj = Xb + (i64)j * nin;
                for (int a = 0; a < nin; ++a) yo[a] = yo[a] + (hij * corx[a]) * xj[a];
            }
        }
    }
}

/* H3X (matrix.f90:188-203): per-point matrices of the outermost layer,
 *   Y(:,i) = sum_j A(:,i,j) X(:,j). */
void orc_h3x(int nin, int nout, const double *A, const double *X, double *Y)
{
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nout; ++i) {
        double *yo = Y + (i64)i * nin;
        const double *a0 = A + (i64)i * nin;
        for (int a = 0; a < nin; ++a) yo[a] = a0[a] * X[a];
        for (int j = 1; j < nout; ++j) {
            const double *aij = A + (i64)nin * (i + (i64)j * nout);
            const double *xj = X + (i64)j * nin;
            for (int a = 0; a < nin; ++a) yo[a] = yo[a] + aij[a] * xj[a];
        }
    }
}

/* VX / VTX (hpx.f90:40-73): in-place rotation of each block by its own
 * nout x nout matrix V(:,:,b) (VX) or its transpose (VTX). */
static void vx_impl(int nin, int nout, int blk, const double *V, double *X, int trans)
{
    #pragma omp parallel
    {
        double *tmp = (double *)malloc(sizeof(double) * (size_t)nin * nout);
        #pragma omp for schedule(static)
        for (int b = 0; b < blk; ++b) {
            const double *Vb = V + (i64)b * nout * nout;
            double *Xb = X + (i64)b * nin * nout;
            for (int i = 0; i < nout; ++i) {
                double *to = tmp + (i64)i * nin;
                const double v0 = trans ? Vb[(i64)i * nout] : Vb[i];
                for (int a = 0; a < nin; ++a) to[a] = v0 * Xb[a];
                for (int j = 1; j < nout; ++j) {
                    const double v = trans ? Vb[j + (i64)i * nout] : Vb[i + (i64)j * nout];
                    const double *xj = Xb + (i64)j * nin;
                    for (int a = 0; a < nin; ++a) to[a] = to[a] + v * xj[a];
                }
            }
            memcpy(Xb, tmp, sizeof(double) * (size_t)nin * nout);
        }
        free(tmp);
    }
}

void orc_vx(int nin, int nout, int blk, const double *V, double *X) { vx_impl(nin, nout, blk, V, X, 0); }
void orc_vtx(int nin, int nout, int blk, const double *V, double *X) { vx_impl(nin, nout, blk, V, X, 1); }

/* ---------------------------------------------------------------------------
 * Whole operator.  Layout and sizes: calOSB (src/iterate/module/osb.init.h:2-49).
 * ------------------------------------------------------------------------- */
typedef struct {
    int sF;
    int sN[ORC_FMAX];
    int sDEP[ORC_FMAX];
    int sNDVR;
    const double *H0;    /* concatenated level matrices (myH0) */
    const double *RES;   /* diagonal potential, length myLen */
    const double *DEP;   /* concatenated myDim(l) factors of dependent levels (myDEP) */
    const double *OUTH;  /* outermost-layer per-point matrices when sNDVR */
    double E0;           /* sOSBW%mE0 */
} orc_osb;

static void layout(const orc_osb *o, i64 *dim, i64 *blk, i64 *h0s, i64 *deps, i64 *len)
{
    dim[0] = 1;
    for (int i = 0; i < o->sF - 1; ++i) dim[i + 1] = dim[i] * o->sN[i];
    blk[o->sF - 1] = 1;
    for (int i = o->sF - 1; i >= 1; --i) blk[i - 1] = blk[i] * o->sN[i];
    *len = blk[0] * o->sN[0];
    i64 s = 0, d = 0;
    for (int i = 0; i < o->sF; ++i) {
        h0s[i] = s;
        if (!(o->sNDVR && i == o->sF - 1)) s += (i64)o->sN[i] * o->sN[i];
        deps[i] = d;
        if (o->sDEP[i]) d += dim[i];
    }
}

/* MYHX (src/iterate/module/osb.hx.h:71-110):
 *   Y = (RES - E0 [ntype != 0]) * X, then for level = 1..sF: Y = Y + H_level X. */
void orc_myhx(const orc_osb *o, int ntype, const double *X, double *Y, double *tmp)
{
    i64 dim[ORC_FMAX], blk[ORC_FMAX], h0s[ORC_FMAX], deps[ORC_FMAX], len;
    layout(o, dim, blk, h0s, deps, &len);
    const double e0 = (ntype == 0) ? 0.0 : o->E0;
    if (ntype == 0) {
        #pragma omp parallel for schedule(static)
        for (i64 p = 0; p < len; ++p) Y[p] = o->RES[p] * X[p];
    } else {
        #pragma omp parallel for schedule(static)
        for (i64 p = 0; p < len; ++p) Y[p] = (o->RES[p] - e0) * X[p];
    }
    for (int l = 0; l < o->sF; ++l) {
        if (o->sNDVR && l == o->sF - 1)
            orc_h3x((int)dim[l], o->sN[l], o->OUTH, X, tmp);
        else if (o->sDEP[l])
            orc_h1x_dep((int)dim[l], o->sN[l], (int)blk[l], o->H0 + h0s[l], o->DEP + deps[l], X, tmp);
        else
            orc_h1x_xyz((int)dim[l], o->sN[l], (int)blk[l], o->H0 + h0s[l], X, tmp);
        #pragma omp parallel for schedule(static)
        for (i64 p = 0; p < len; ++p) Y[p] = Y[p] + tmp[p];
    }
}

/* MYPX (src/iterate/module/osb.px.h:125-219) for the TOSB, TOSBD1 and TOSBD2
 * kernels: Y = V_sF..V_1 K^-1 V_1^T..V_sF^T X.  npc == 0 uses E0 = 0 (TA0). */
int orc_mypx(const orc_osb *o, const double *VOSB, const double *EIG0, int nosb, int npc,
             double de, double beta_in, const double *X, double *Y)
{
    i64 dim[ORC_FMAX], blk[ORC_FMAX], h0s[ORC_FMAX], deps[ORC_FMAX], len;
    layout(o, dim, blk, h0s, deps, &len);
    i64 vs[ORC_FMAX], v = 0;
    for (int l = 0; l < o->sF; ++l) { vs[l] = v; v += blk[l] * (i64)o->sN[l] * o->sN[l]; }
    memcpy(Y, X, sizeof(double) * (size_t)len);
    const double DE = fabs(de), RDE = 1.0 / DE;
    for (int l = o->sF - 1; l >= 0; --l)
        orc_vtx((int)dim[l], o->sN[l], (int)blk[l], VOSB + vs[l], Y);
    const double E0 = (npc == 0) ? 0.0 : o->E0;
    switch (nosb) {
    case 2: /* TOSBD1 (osb.px.h:160-172) */
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < len; ++i) {
            const double ade = EIG0[i] - E0;
            if (fabs(ade) <= DE) Y[i] = (ade < 0.0) ? -Y[i] * RDE : Y[i] * RDE;
            else Y[i] = Y[i] / ade;
        }
        break;
    case 3: { /* TOSBD2 (osb.px.h:174-189) */
        const double beta = 1.0 + beta_in, alpha = -beta_in * DE;
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < len; ++i) {
            const double ade = EIG0[i] - E0;
            double t;
            if (fabs(ade) <= DE) t = (ade < 0.0) ? (-alpha + beta * ade) : (alpha + beta * ade);
            else t = ade;
            Y[i] = Y[i] / t;
        }
        break;
    }
    case 4:
        return -1; /* TOSBW (window LDL^T) is not restated */
    default: /* TOSB (osb.px.h:156-158) */
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < len; ++i) Y[i] = Y[i] / (EIG0[i] - E0);
        break;
    }
    for (int l = 0; l < o->sF; ++l)
        orc_vx((int)dim[l], o->sN[l], (int)blk[l], VOSB + vs[l], Y);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Block-Jacobi build of the OSB preconditioner.
 * ------------------------------------------------------------------------- */

/* HOSBINIT_XYZ (src/iterate/libiterate/diag/hinitxyz.f90:7-29). */
void orc_hosbinit_xyz(int blk, int mak, int ndk, const double *H1, const double *RES, double *HOSB)
{
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b)
        for (int j = 0; j < mak; ++j)
            for (int k = 0; k < mak; ++k) {
                double *h = HOSB + (i64)ndk * (k + (i64)mak * (j + (i64)mak * b));
                const double v = H1[k + (i64)j * mak];
                for (int a = 0; a < ndk; ++a) h[a] = v;
            }
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b)
        for (int k = 0; k < mak; ++k) {
            double *h = HOSB + (i64)ndk * (k + (i64)mak * (k + (i64)mak * b));
            const double *r = RES + (i64)ndk * (k + (i64)mak * b);
            for (int a = 0; a < ndk; ++a) h[a] = h[a] + r[a];
        }
}

/* HOSBINIT_DEP (src/iterate/libiterate/diag/hinitdep.f90:10-34). */
void orc_hosbinit_dep(int blk, int mak, int ndk, const double *H1, const double *DEP,
                      const double *RES, double *HOSB)
{
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b)
        for (int j = 0; j < mak; ++j)
            for (int k = 0; k < mak; ++k) {
                double *h = HOSB + (i64)ndk * (k + (i64)mak * (j + (i64)mak * b));
                const double v = H1[k + (i64)j * mak];
                for (int a = 0; a < ndk; ++a) h[a] = v * DEP[a];
            }
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < blk; ++b)
        for (int k = 0; k < mak; ++k) {
            double *h = HOSB + (i64)ndk * (k + (i64)mak * (k + (i64)mak * b));
            const double *r = RES + (i64)ndk * (k + (i64)mak * b);
            for (int a = 0; a < ndk; ++a) h[a] = h[a] + r[a];
        }
}

static double dot_seq(i64 n, const double *x, const double *y)
{
    double s = 0.0;
    for (i64 i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

/* sumOffDiag (src/iterate/libiterate/diag/sumdiag.f90:6-22). */
double orc_sumoffdiag(int nin, int nout, const double *H)
{
    double s = 0.0;
    for (int i = 0; i < nout; ++i)
        for (int j = 0; j < i; ++j) {
            const double *h = H + (i64)nin * (j + (i64)nout * i);
            s = s + dot_seq(nin, h, h);
        }
    return 2.0 * s;
}

/* sumDiag (sumdiag.f90:28-41). */
double orc_sumdiag(int nin, int nout, const double *H)
{
    double s = 0.0;
    for (int i = 0; i < nout; ++i) {
        const double *h = H + (i64)nin * (i + (i64)nout * i);
        s = s + dot_seq(nin, h, h);
    }
    return s;
}

/* MJACOBI (src/iterate/libiterate/diag/jacobi.f90:2-83): one joint Jacobi
 * rotation of the (p,q) plane of all nin stacked nout x nout matrices.
 * p, q are 1-based as in the reference.  Returns the rotation angle. */
double orc_mjacobi(int P, int Q, int nout, int nin, double *H, double *work)
{
    const double PIE = 3.14159265358979323846264338328;
    const int p = P - 1, q = Q - 1;
    double *ddg = work, *odg = work + nin;
    double *hpp = H + (i64)nin * (p + (i64)nout * p);
    double *hqq = H + (i64)nin * (q + (i64)nout * q);
    double *hpq = H + (i64)nin * (p + (i64)nout * q);
    double *hqp = H + (i64)nin * (q + (i64)nout * p);
    for (int a = 0; a < nin; ++a) {
        odg[a] = hpq[a];
        ddg[a] = 0.5 * hpp[a] - 0.5 * hqq[a];
    }
    const double A = dot_seq(nin, odg, odg);
    const double B = 2.0 * dot_seq(nin, odg, ddg);
    const double C = dot_seq(nin, ddg, ddg);
    double X;
    if (A == C) {
        if (B == 0.0) X = 0.0;
        else X = -copysign(PIE / 8.0, B);
    } else {
        X = atan(B / (A - C)) / 4.0;
        if (A > C) {
            if (X < 0.0) X = X + PIE / 4.0;
            else X = X - PIE / 4.0;
        }
    }
    const double SN = sin(X), CS = cos(X);
    const double C2 = CS * CS, S2 = SN * SN, SC = SN * CS;
    #pragma omp parallel for schedule(static) if (nin > 4096)
    for (int a = 0; a < nin; ++a) {
        const double np_ = C2 * hpp[a] + S2 * hqq[a] - 2 * SC * odg[a];
        const double nq_ = C2 * hqq[a] + S2 * hpp[a] + 2 * SC * odg[a];
        const double nqp = (C2 - S2) * odg[a] + 2 * SC * ddg[a];
        hpp[a] = np_;
        hqq[a] = nq_;
        hpq[a] = nqp;
        hqp[a] = nqp;
    }
    for (int r = 0; r < nout; ++r) {
        if (r == p || r == q) continue;
        double *hrp = H + (i64)nin * (r + (i64)nout * p);
        double *hrq = H + (i64)nin * (r + (i64)nout * q);
        double *hpr = H + (i64)nin * (p + (i64)nout * r);
        double *hqr = H + (i64)nin * (q + (i64)nout * r);
        #pragma omp parallel for schedule(static) if (nin > 4096)
        for (int a = 0; a < nin; ++a) {
            const double np_ = CS * hrp[a] - SN * hrq[a];
            const double nq_ = CS * hrq[a] + SN * hrp[a];
            hrp[a] = np_;
            hpr[a] = np_;
            hrq[a] = nq_;
            hqr[a] = nq_;
        }
    }
    return X;
}

/* VINIT / VUPDATE (src/iterate/libiterate/diag/vupdate.f90:4-36). */
void orc_vinit(int nout, double *V)
{
    memset(V, 0, sizeof(double) * (size_t)nout * nout);
    for (int i = 0; i < nout; ++i) V[i + (i64)i * nout] = 1.0;
}

void orc_vupdate(int P, int Q, double phi, int nout, double *V)
{
    const double c = cos(phi), s = sin(phi);
    double *vp = V + (i64)(P - 1) * nout, *vq = V + (i64)(Q - 1) * nout;
    for (int a = 0; a < nout; ++a) {
        const double t = c * vp[a] - s * vq[a];
        vq[a] = c * vq[a] + s * vp[a];
        vp[a] = t;
    }
}

/* HosbDiag (src/iterate/libiterate/diag/hosbdiag.f90:5-75).  stats (optional,
 * length 5) receives the reference's eff(1:5) accumulators; sweeps (optional,
 * length blk) the sweep count k-1 of every block. */
void orc_hosbdiag(int bjmax, double bjtol, int blk, int mak, int ndk, double *HOSB,
                  double *VOSB, double *EIGVAL, double *stats, int *sweeps)
{
    double eff[5] = {INFINITY, -INFINITY, 0, 0, 0};
    const int inner_par = (blk == 1);
    #pragma omp parallel for schedule(dynamic, 1) if (!inner_par)
    for (int it = 0; it < blk; ++it) {
        double *H = HOSB + (i64)ndk * mak * mak * it;
        double *V = VOSB + (i64)mak * mak * it;
        double *work = (double *)malloc(sizeof(double) * 2 * (size_t)ndk);
        const double initye = orc_sumoffdiag(ndk, mak, H);
        double ye = initye, dye = initye;
        int k = 1;
        orc_vinit(mak, V);
        while (fabs(dye) > initye * bjtol && k <= bjmax) {
            for (int i = 1; i <= mak - 1; ++i)
                for (int j = 1; j <= mak - i; ++j) {
                    const double phi = orc_mjacobi(j, j + i, mak, ndk, H, work);
                    orc_vupdate(j, j + i, phi, mak, V);
                }
            dye = orc_sumoffdiag(ndk, mak, H) - ye;
            ye = ye + dye;
            k = k + 1;
        }
        free(work);
        if (sweeps) sweeps[it] = k - 1;
        const double eff0 = fabs(1.0 - ye / initye);
        const double sd = orc_sumdiag(ndk, mak, H);
        for (int i = 0; i < mak; ++i) {
            double *hii = H + (i64)ndk * (i + (i64)mak * i);
            double *e = EIGVAL + (i64)ndk * (i + (i64)mak * it);
            for (int a = 0; a < ndk; ++a) e[a] = hii[a];
            for (int a = 0; a < ndk; ++a) hii[a] = 0.0;
        }
        #pragma omp critical
        {
            if (eff0 < eff[0]) eff[0] = eff0;
            if (eff0 > eff[1]) eff[1] = eff0;
            eff[2] += eff0; eff[3] += sd; eff[4] += k;
        }
    }
    if (stats) memcpy(stats, eff, sizeof(eff));
}

/* myDiag (src/iterate/module/osb.diag.h:53-151) with myDiagInit
 * (osb.diag.h:18-31, osb.diag.init.h): level sF..1, EIG0 in/out (in: RES). */
int orc_mydiag(const orc_osb *o, int bjmax, double bjtol, double *VOSB, double *EIG0,
               double *stats /* 5*sF or NULL */)
{
    i64 dim[ORC_FMAX], blk[ORC_FMAX], h0s[ORC_FMAX], deps[ORC_FMAX], len;
    layout(o, dim, blk, h0s, deps, &len);
    i64 vs[ORC_FMAX], v = 0, hmax = 0;
    for (int l = 0; l < o->sF; ++l) {
        vs[l] = v;
        v += blk[l] * (i64)o->sN[l] * o->sN[l];
        if ((i64)o->sN[l] * len > hmax) hmax = (i64)o->sN[l] * len;
    }
    double *HOSB = (double *)malloc(sizeof(double) * (size_t)hmax);
    if (!HOSB) return -1;
    for (int l = o->sF - 1; l >= 0; --l) {
        if (o->sNDVR && l == o->sF - 1)
            memcpy(HOSB, o->OUTH, sizeof(double) * (size_t)(o->sN[l] * len));
        else if (o->sDEP[l])
            orc_hosbinit_dep((int)blk[l], o->sN[l], (int)dim[l], o->H0 + h0s[l], o->DEP + deps[l], EIG0, HOSB);
        else
            orc_hosbinit_xyz((int)blk[l], o->sN[l], (int)dim[l], o->H0 + h0s[l], EIG0, HOSB);
        orc_hosbdiag(bjmax, bjtol, (int)blk[l], o->sN[l], (int)dim[l], HOSB, VOSB + vs[l], EIG0,
                     stats ? stats + 5 * l : NULL, NULL);
    }
    free(HOSB);
    return 0;
}

/* ---------------------------------------------------------------------------
 * QMR (src/iterate/libiterate/qmr/qmr.f90:5-175; breakdown codes as QMR_MPI,
 * src/iterate/libiterate_mpi/qmr/qmr_mpi.f90:4-263, when mpi_codes != 0).
 * ------------------------------------------------------------------------- */
typedef void (*orc_op)(void *ctx, int n, const double *x, double *y);

static double dotp(int n, const double *x, const double *y) { return dot_seq(n, x, y); }

int orc_qmr(int ntype, int qmrmax, double qmrtol, int n, const double *B,
            orc_op hx, void *hctx, orc_op px, void *pctx, double *X, double *res,
            int mpi_codes, int *iters_out)
{
    double *R = malloc(sizeof(double) * (size_t)n), *UX = malloc(sizeof(double) * (size_t)n);
    double *UR = malloc(sizeof(double) * (size_t)n), *Q = malloc(sizeof(double) * (size_t)n);
    double *S = malloc(sizeof(double) * (size_t)n), *V = malloc(sizeof(double) * (size_t)n);
    double *Z = malloc(sizeof(double) * (size_t)n), *HX0 = malloc(sizeof(double) * (size_t)n);
    double BNRM, ZNRM, VNRM, VNRMPO = 0, ZVRAT, QSDOT = 1, VZDOT, BETA, ETA;
    double GAMAMO, GAMA, THETAMO = 0, THETA;
    int qmr = -1, i;
    *res = 0.0;
    ZVRAT = 1.0;
    if (ntype <= 0) memset(X, 0, sizeof(double) * (size_t)n);
    memcpy(R, B, sizeof(double) * (size_t)n);
    memcpy(V, B, sizeof(double) * (size_t)n);
    BNRM = sqrt(dotp(n, B, B));
    VNRM = BNRM;
    px(pctx, n, B, Z);
    ZNRM = sqrt(dotp(n, Z, Z));
    GAMAMO = 1.0; ETA = -1.0;
    qmr = 0;
    for (i = 1; i <= qmrmax; ++i) {
        if (VNRM == 0.0 || ZNRM == 0.0) { if (mpi_codes) qmr = -1; break; }
        ZVRAT = ZVRAT * ZNRM / VNRM;
        for (int k = 0; k < n; ++k) { V[k] = V[k] / VNRM; Z[k] = Z[k] / ZNRM; }
        VZDOT = dotp(n, V, Z);
        if (VZDOT == 0.0) { if (mpi_codes) qmr = -2; break; }
        if (i == 1) memcpy(Q, Z, sizeof(double) * (size_t)n);
        else {
            const double f = VNRM * VZDOT / QSDOT;
            for (int k = 0; k < n; ++k) Q[k] = Z[k] - f * Q[k];
        }
        hx(hctx, n, Q, S);
        for (int k = 0; k < n; ++k) S[k] = ZVRAT * S[k];
        QSDOT = dotp(n, Q, S);
        BETA = QSDOT / VZDOT;
        if (QSDOT == 0.0 || BETA == 0.0) { if (mpi_codes) qmr = -3; break; }
        for (int k = 0; k < n; ++k) V[k] = S[k] - BETA * V[k];
        VNRMPO = sqrt(dotp(n, V, V));
        px(pctx, n, V, Z);
        for (int k = 0; k < n; ++k) Z[k] = Z[k] / ZVRAT;
        ZNRM = sqrt(dotp(n, Z, Z));
        THETA = VNRMPO / (GAMAMO * fabs(BETA));
        GAMA = 1.0 / sqrt(1.0 + THETA * THETA);
        ETA = -ETA * VNRM * GAMA * GAMA / (BETA * GAMAMO * GAMAMO);
        if (GAMA == 0.0) { if (mpi_codes) qmr = -4; break; }
        if (i == 1) {
            const double f = ETA * ZVRAT;
            for (int k = 0; k < n; ++k) { UX[k] = f * Q[k]; UR[k] = ETA * S[k]; }
        } else {
            const double f = ETA * ZVRAT, g = (THETAMO * GAMA) * (THETAMO * GAMA);
            for (int k = 0; k < n; ++k) {
                UX[k] = f * Q[k] + g * UX[k];
                UR[k] = ETA * S[k] + g * UR[k];
            }
        }
        for (int k = 0; k < n; ++k) { X[k] = X[k] + UX[k]; R[k] = R[k] - UR[k]; }
        double RES;
        switch (abs(ntype)) {
        case 1: {
            hx(hctx, n, X, HX0);
            const double XNRM = sqrt(dotp(n, HX0, HX0));
            for (int k = 0; k < n; ++k) HX0[k] = HX0[k] - B[k];
            RES = sqrt(dotp(n, HX0, HX0)) / XNRM;
            break;
        }
        case 2: {
            const double r1 = sqrt(dotp(n, R, R)) / BNRM;
            const double r2 = sqrt(dotp(n, UX, UX) / dotp(n, X, X));
            const double r3 = sqrt(dotp(n, UR, UR) / dotp(n, R, R));
            RES = r1 > r2 ? r1 : r2;
            RES = RES > r3 ? RES : r3;
            break;
        }
        default:
            RES = sqrt(dotp(n, R, R)) / BNRM;
        }
        *res = RES;
        if (fabs(RES) < qmrtol) { qmr = i; break; }
        qmr = -i;
        VNRM = VNRMPO; GAMAMO = GAMA; THETAMO = THETA;
    }
    if (iters_out) *iters_out = (i > qmrmax) ? qmrmax : i;
    free(R); free(UX); free(UR); free(Q); free(S); free(V); free(Z); free(HX0);
    return qmr;
}

/* Operator adaptors usable as orc_op callbacks. */
typedef struct { const orc_osb *o; int ntype; double *tmp; } orc_hx_ctx;
typedef struct { const orc_osb *o; const double *VOSB; const double *EIG0; int nosb; int npc;
                 double de; double beta; } orc_px_ctx;

void orc_hx_op(void *ctx, int n, const double *x, double *y)
{
    (void)n;
    orc_hx_ctx *c = (orc_hx_ctx *)ctx;
    orc_myhx(c->o, c->ntype, x, y, c->tmp);
}

void orc_px_op(void *ctx, int n, const double *x, double *y)
{
    (void)n;
    orc_px_ctx *c = (orc_px_ctx *)ctx;
    orc_mypx(c->o, c->VOSB, c->EIG0, c->nosb, c->npc, c->de, c->beta, x, y);
}

/* Dense symmetric matrix (column-major) and its Jacobi preconditioner, the
 * operators of the reference's QMR unit driver (qmr.drv.f90:56-119). */
typedef struct { int n; const double *H; } orc_dense_ctx;

void orc_dense_hx(void *ctx, int n, const double *x, double *y)
{
    orc_dense_ctx *c = (orc_dense_ctx *)ctx;
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s = s + c->H[i + (i64)j * c->n] * x[j];
        y[i] = s;
    }
}

void orc_dense_jacobi_px(void *ctx, int n, const double *x, double *y)
{
    orc_dense_ctx *c = (orc_dense_ctx *)ctx;
    for (int i = 0; i < n; ++i) y[i] = x[i] / c->H[i + (i64)i * c->n];
}

/* QMR on the whole OSB operator pair (OSB_QMR, src/iterate/module/osbw.qmr.h:13-23):
 * HX = MYHX(TA1), PX = MYPX(nosb, TA1). */
int orc_osb_qmr(const orc_osb *o, const double *VOSB, const double *EIG0, int nosb, double de,
                double beta, int ntype, int qmrmax, double qmrtol, const double *B, double *X,
                double *res, int mpi_codes, int *iters_out)
{
    i64 dim[ORC_FMAX], blk[ORC_FMAX], h0s[ORC_FMAX], deps[ORC_FMAX], len;
    layout(o, dim, blk, h0s, deps, &len);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)len);
    orc_hx_ctx hc = {o, 1, tmp};
    orc_px_ctx pc = {o, VOSB, EIG0, nosb, 1, de, beta};
    int r = orc_qmr(ntype, qmrmax, qmrtol, (int)len, B, orc_hx_op, &hc, orc_px_op, &pc, X, res,
                    mpi_codes, iters_out);
    free(tmp);
    return r;
}

/* MGS_ORTH (src/iterate/libiterate/orth/gsorth.f90:42-72): orthogonalise W
 * against the m columns of VJ (leading dimension n) into column m (0-based). */
int orc_mgs_orth(int n, const double *W, int m, double *VJ)
{
    double *v = VJ + (i64)n * m;
    memcpy(v, W, sizeof(double) * (size_t)n);
    const double normw = sqrt(dot_seq(n, W, W));
    if (normw == 0.0) return 0;
    for (int i = 0; i < m; ++i) {
        const double *u = VJ + (i64)n * i;
        const double d = dot_seq(n, v, u);
        for (int k = 0; k < n; ++k) v[k] = v[k] - d * u[k];
    }
    const double nrm = sqrt(dot_seq(n, v, v));
    if (nrm == 0.0) return 0;
    for (int k = 0; k < n; ++k) v[k] = v[k] / nrm;
    return 1;
}

/* Sequential FP64 dot, exported so the Python side of the oracle can build
 * HMAT with the reference's summation order (pistHij.f90:117-123). */
double orc_dot(i64 n, const double *x, const double *y) { return dot_seq(n, x, y); }

int orc_num_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
