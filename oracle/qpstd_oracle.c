/*
 * qpstd_oracle.c -- FP64 CPU oracle (TEST INFRASTRUCTURE ONLY, see the header).
 *
 * Everything here is double precision and deliberately literal: 2-D C2C
 * transforms, complex intermediates, and the same kernel order as the
 * reference's GPU drivers.  Each function names the reference lines it follows.
 */
#include "qpstd_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* The reference's host code defines pi as 3.1415926 (sgpstd-qmodeling/funca.c:6,
 * statement.h:7); the coefficient tables inherit that constant. */
#define REF_PI 3.1415926

/* ======================================================================== */
/* 1-D FFT: Stockham mixed radix for factors <= 13, Bluestein otherwise.      */
/* ======================================================================== */

typedef struct fftp {
    int n, nst, rad[64];
    cplx *w;                  /* w[m] = exp(-2 pi i m / n) */
    int blue, m;
    struct fftp *sub;         /* length-m plan for Bluestein */
    cplx *chirp;              /* exp(-i pi k^2 / n) */
    cplx *bhat;               /* FFT_m of the wrapped conj chirp */
} fftp;

static fftp *fft_plan(int n);
static void fft_exec(const fftp *p, cplx *x, cplx *scratch, int sign);

static int smooth7(int v) {
    while (v % 2 == 0) v /= 2;
    while (v % 3 == 0) v /= 3;
    while (v % 5 == 0) v /= 5;
    while (v % 7 == 0) v /= 7;
    return v == 1;
}

static fftp *fft_plan(int n) {
    fftp *p = (fftp *)calloc(1, sizeof(fftp));
    p->n = n;
    p->w = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int m = 0; m < n; m++) {
        double a = -2.0 * M_PI * (double)m / (double)n;
        p->w[m] = cos(a) + I * sin(a);
    }
    int v = n, big = 0;
    while (v % 4 == 0) { p->rad[p->nst++] = 4; v /= 4; }
    while (v % 2 == 0) { p->rad[p->nst++] = 2; v /= 2; }
    for (int f = 3; f * f <= v || f <= v; f += 2) {
        while (v % f == 0) {
            if (f > 13) big = 1;
            p->rad[p->nst++] = f;
            v /= f;
        }
        if (v == 1) break;
    }
    if (big) {
        p->blue = 1;
        int m = 2 * n - 1;
        while (!smooth7(m)) m++;
        p->m = m;
        p->sub = fft_plan(m);
        p->chirp = (cplx *)malloc(sizeof(cplx) * (size_t)n);
        for (long long k = 0; k < n; k++) {
            long long q = (k * k) % (2LL * n);
            double a = -M_PI * (double)q / (double)n;
            p->chirp[k] = cos(a) + I * sin(a);
        }
        p->bhat = (cplx *)calloc((size_t)m, sizeof(cplx));
        for (int k = 0; k < n; k++) p->bhat[k] = conj(p->chirp[k]);
        for (int k = 1; k < n; k++) p->bhat[m - k] = conj(p->chirp[k]);
        cplx *s = (cplx *)malloc(sizeof(cplx) * (size_t)(2 * m));
        fft_exec(p->sub, p->bhat, s, -1);
        free(s);
    }
    return p;
}

static void fft_free(fftp *p) {
    if (!p) return;
    free(p->w);
    if (p->blue) { fft_free(p->sub); free(p->chirp); free(p->bhat); }
    free(p);
}

/* scratch: >= 2*n (Stockham) or 2*m + m (Bluestein) complex values */
static void fft_exec(const fftp *p, cplx *x, cplx *scratch, int sign) {
    const int n = p->n;
    if (n == 1) return;
    if (p->blue) {
        const int m = p->m;
        cplx *a = scratch, *s2 = scratch + m;
        if (sign > 0) for (int k = 0; k < n; k++) x[k] = conj(x[k]);
        for (int k = 0; k < n; k++) a[k] = x[k] * p->chirp[k];
        for (int k = n; k < m; k++) a[k] = 0;
        fft_exec(p->sub, a, s2, -1);
        for (int k = 0; k < m; k++) a[k] *= p->bhat[k];
        fft_exec(p->sub, a, s2, +1);
        for (int k = 0; k < n; k++) x[k] = p->chirp[k] * a[k] / (double)m;
        if (sign > 0) for (int k = 0; k < n; k++) x[k] = conj(x[k]);
        return;
    }
    cplx *src = x, *dst = scratch;
    int ns = 1;
    cplx v[16], out[16];
    for (int st = 0; st < p->nst; st++) {
        const int r = p->rad[st];
        const int nr = n / r;
        const int stride = n / (ns * r);
        for (int j = 0; j < nr; j++) {
            const int k = j % ns;
            for (int q = 0; q < r; q++) {
                cplx t = p->w[q * k * stride];
                if (sign > 0) t = conj(t);
                v[q] = src[j + q * nr] * t;
            }
            for (int q = 0; q < r; q++) {
                cplx acc = 0;
                for (int u = 0; u < r; u++) {
                    cplx t = p->w[((u * q) % r) * nr];
                    if (sign > 0) t = conj(t);
                    acc += v[u] * t;
                }
                out[q] = acc;
            }
            const int base = (j / ns) * ns * r + k;
            for (int q = 0; q < r; q++) dst[base + q * ns] = out[q];
        }
        cplx *t = src; src = dst; dst = t;
        ns *= r;
    }
    if (src != x) memcpy(x, src, sizeof(cplx) * (size_t)n);
}

static size_t fft_scratch_len(const fftp *p) {
    return p->blue ? (size_t)(3 * p->m) : (size_t)(2 * p->n);
}

int orc_fft1d(int n, double *re_im, int sign) {
    if (n < 1) return -1;
    fftp *p = fft_plan(n);
    cplx *x = (cplx *)re_im;
    cplx *s = (cplx *)malloc(sizeof(cplx) * fft_scratch_len(p));
    fft_exec(p, x, s, sign);
    free(s);
    fft_free(p);
    return 0;
}

/* 2-D C2C transform of an x-major nxx*nzz array (cufftPlan2d(nxx,nzz) layout,
 * sgpstd-qmodeling/acps4.cu:871).  Unnormalised. */
typedef struct { fftp *px, *pz; int nxx, nzz; } fft2;

static void fft2_exec(const fft2 *f, cplx *a, int sign) {
    const int nxx = f->nxx, nzz = f->nzz;
#pragma omp parallel
    {
        size_t sl = fft_scratch_len(f->pz);
        size_t sx = fft_scratch_len(f->px);
        cplx *s = (cplx *)malloc(sizeof(cplx) * (sl > sx ? sl : sx));
        cplx *col = (cplx *)malloc(sizeof(cplx) * (size_t)nxx);
#pragma omp for schedule(static)
        for (int ix = 0; ix < nxx; ix++) fft_exec(f->pz, a + (size_t)ix * nzz, s, sign);
#pragma omp for schedule(static)
        for (int iz = 0; iz < nzz; iz++) {
            for (int ix = 0; ix < nxx; ix++) col[ix] = a[(size_t)ix * nzz + iz];
            fft_exec(f->px, col, s, sign);
            for (int ix = 0; ix < nxx; ix++) a[(size_t)ix * nzz + iz] = col[ix];
        }
        free(col);
        free(s);
    }
}

/* ======================================================================== */
/* Coefficient setup (FP64 restatements of the reference host functions).   */
/* ======================================================================== */

/* CPML profiles: sgpstd-qmodeling/funca.c:223-340 (get_pml_parameters). */
void orc_pml_coeffs(int pml, double fm, int nxx, int nzz, double dx, double dz, double dt,
                    double *i_ax, double *i_bx, double *i_az, double *i_bz,
                    double *h_ax, double *h_bx, double *h_az, double *h_bz) {
    const double alpha_max = REF_PI * fm, R = 1e-5, vmax = 5000.0;
    const int n1 = 2, n2 = 1, n3 = 1;
    double *idx = calloc(nxx, 8), *idz = calloc(nzz, 8), *iax = calloc(nxx, 8), *iaz = calloc(nzz, 8);
    double *hdx = calloc(nxx, 8), *hdz = calloc(nzz, 8), *hax = calloc(nxx, 8), *haz = calloc(nzz, 8);
    const double dmaxx = (1 + n1 + n2) * vmax * log(1.0 / R) / (2.0 * pml * dx);
    const double dmaxz = (1 + n1 + n2) * vmax * log(1.0 / R) / (2.0 * pml * dz);
    for (int i = 0; i < pml; i++) {
        double t1 = pow((double)(pml - 1 - i) / pml, n1 + n2);
        double t3 = pow((double)i / (pml - 1), n3);
        idx[i] = dmaxx * t1; idz[i] = dmaxz * t1;
        iax[i] = alpha_max * t3; iaz[i] = iax[i];
        idx[nxx - 1 - i] = idx[i]; idz[nzz - 1 - i] = idz[i];
        iax[nxx - 1 - i] = iax[i]; iaz[nzz - 1 - i] = iaz[i];
    }
    for (int i = pml; i < nxx - pml; i++) { idx[i] = 0; iax[i] = iax[pml - 1]; }
    for (int j = pml; j < nzz - pml; j++) { idz[j] = 0; iaz[j] = iaz[pml - 1]; }
    for (int i = 0; i < pml - 1; i++) {
        double t2 = pow((pml - 1.5 - i) / pml, n1 + n2);
        double t4 = pow((i + 0.5) / (pml - 1), n3);
        hdx[i] = dmaxx * t2; hdz[i] = dmaxz * t2;
        hdx[nxx - 2 - i] = hdx[i]; hdz[nzz - 2 - i] = hdz[i];
        hax[i] = alpha_max * t4; haz[i] = hax[i];
        hax[nxx - 2 - i] = hax[i]; haz[nzz - 2 - i] = haz[i];
    }
    for (int i = pml - 1; i < nxx - pml; i++) { hdx[i] = 0; hax[i] = hax[pml - 2]; }
    hdx[nxx - 1] = 0; hax[nxx - 1] = hax[nxx - 2];
    for (int j = pml - 1; j < nzz - pml; j++) { hdz[j] = 0; haz[j] = haz[pml - 2]; }
    hdz[nzz - 1] = 0; haz[nzz - 1] = haz[nzz - 2];
    for (int i = 0; i < nxx; i++) {
        double t = idx[i] + iax[i];
        i_bx[i] = exp(-dt * t); i_ax[i] = idx[i] / t * (i_bx[i] - 1.0);
        t = hdx[i] + hax[i];
        h_bx[i] = exp(-dt * t); h_ax[i] = hdx[i] / t * (h_bx[i] - 1.0);
    }
    for (int j = 0; j < nzz; j++) {
        double t = idz[j] + iaz[j];
        i_bz[j] = exp(-dt * t); i_az[j] = idz[j] / t * (i_bz[j] - 1.0);
        t = hdz[j] + haz[j];
        h_bz[j] = exp(-dt * t); h_az[j] = hdz[j] / t * (h_bz[j] - 1.0);
    }
    free(idx); free(idz); free(iax); free(iaz); free(hdx); free(hdz); free(hax); free(haz);
}

/* wavenumber magnitude as the reference builds it (funca.c:366-381) */
static double kk_of(int i, int n, double d) {
    const double dk = 2.0 * REF_PI / (n * d);
    const int nh = n / 2 + 1;
    return (i < nh) ? i * dk : (n - i) * dk;
}

/* Half-cell shift tables: sgpstd-qmodeling/funca.c:342-432 (cal_shift_parameters).
 * For odd n the negative-frequency half mirrors index n-1-i (funca.c:397), which
 * the oracle reproduces. */
void orc_shift_tables(int nxx, int nzz, double dx, double dz,
                      double *kxsmr, double *kxscr, double *kzsmr, double *kzscr,
                      double *kxsmi, double *kxsci, double *kzsmi, double *kzsci) {
    double *sxr = malloc(8 * nxx), *sxi = malloc(8 * nxx), *szr = malloc(8 * nzz), *szi = malloc(8 * nzz);
    const int nxh = nxx / 2 + 1, nzh = nzz / 2 + 1;
    for (int i = 0; i < nxx; i++) {
        if (i < nxh) { double t = i * REF_PI / nxx; sxr[i] = cos(t); sxi[i] = sin(t); }
        else { sxr[i] = sxr[nxx / 2 * 2 - i]; sxi[i] = -sxi[nxx / 2 * 2 - i]; }
        double k = kk_of(i, nxx, dx);
        kxsmr[i] = k * sxr[i]; kxsmi[i] = -k * sxi[i];
        kxscr[i] = k * sxr[i]; kxsci[i] = k * sxi[i];
    }
    for (int j = 0; j < nzz; j++) {
        if (j < nzh) { double t = j * REF_PI / nzz; szr[j] = cos(t); szi[j] = sin(t); }
        else { szr[j] = szr[nzz / 2 * 2 - j]; szi[j] = -szi[nzz / 2 * 2 - j]; }
        double k = kk_of(j, nzz, dz);
        kzsmr[j] = k * szr[j]; kzsmi[j] = k * szi[j];
        kzscr[j] = k * szr[j]; kzsci[j] = -k * szi[j];
    }
    free(sxr); free(sxi); free(szr); free(szi);
}

/* Isotropic symbols: sgpstd-qmodeling/func.c:550-585 (cal_k2d). */
void orc_k2d(int nxx, int nzz, double dx, double dz,
             double *k2d1, double *k2d2, double *k2d3, double *k2da) {
    for (int i = 0; i < nxx; i++) {
        double kx = kk_of(i, nxx, dx);
        for (int j = 0; j < nzz; j++) {
            double kz = kk_of(j, nzz, dz);
            size_t is = (size_t)i * nzz + j;
            double k2 = kx * kx + kz * kz;
            if (k2d1) k2d1[is] = k2;
            if (k2d2) k2d2[is] = pow(k2, 1.0 / 32.0);
            if (k2d3) k2d3[is] = pow(k2, 33.0 / 32.0);
            if (k2da) k2da[is] = pow(k2, 0.505);
        }
    }
}

/* Source wavelet: sgpstd-qmodeling/funca.c:201-220 (rik_cal), t0 = 1/fd. */
void orc_ricker(int nt, double dt, double fd, int flag, double *rik) {
    const double t0 = 1.0 / fd;
    for (int i = 0; i < nt; i++) {
        double tt = i * dt - t0;
        if (flag == 2) {
            double a = pow(REF_PI * fd * tt, 2.0);
            rik[i] = (1.0 - 2.0 * a) * exp(-a);
        } else {
            double a = pow(2.0 * REF_PI * fd * tt, 2.0);
            rik[i] = tt * exp(-a);
        }
    }
}

/* Staggered buoyancy: sgpstd-qmodeling/funca.c:169-198 (cal_bbx_bbz). */
void orc_bbx_bbz(int nxx, int nzz, const double *d, double *bbx, double *bbz) {
    for (int j = 0; j < nzz; j++)
        for (int i = 0; i < nxx - 1; i++) {
            size_t is = (size_t)i * nzz + j;
            bbx[is] = 2.0 / (d[is] + d[is + nzz]);
        }
    for (int j = 0; j < nzz; j++) bbx[(size_t)(nxx - 1) * nzz + j] = 1.0 / d[(size_t)(nxx - 1) * nzz + j];
    for (int i = 0; i < nxx; i++)
        for (int j = 0; j < nzz - 1; j++) {
            size_t is = (size_t)i * nzz + j;
            bbz[is] = 2.0 / (d[is] + d[is + 1]);
        }
    for (int i = 0; i < nxx; i++) bbz[(size_t)i * nzz + nzz - 1] = 1.0 / d[(size_t)i * nzz + nzz - 1];
}

/* Q transform: sgpstd-qmodeling/func.c:912-930 (transfermodel). */
void orc_transfermodel(int n, double fd, double fo, const double *vp, const double *qp,
                       double *gam, double *lam, double *vwd, double *tao) {
    const double wd = 2.0 * REF_PI * fd;
    for (int i = 0; i < n; i++) {
        gam[i] = 1.0 / REF_PI / qp[i];
        lam[i] = pow(fd / fo, 2.0 * gam[i]);
        vwd[i] = pow(vp[i] / wd, 1.0 / 16.0);
        tao[i] = lam[i] * vp[i] / qp[i];
    }
}

/* ======================================================================== */
/* Revolve: the binomial checkpointing schedule of Griewank & Walther        */
/* (ACM TOMS 26(1), Algorithm 799), as driven by sgpstd-qrtm/acsglw.cu:470.  */
/* State lives in the struct instead of function-static storage.             */
/* ======================================================================== */

int orc_numforw(int steps, int snaps) {
    if (snaps < 1 || snaps > 64) return -1;
    int reps = 0, range = 1;
    while (range < steps) { reps++; range = range * (reps + snaps) / reps; }
    if (reps > 64) return -1;
    return reps * steps - range * reps / (snaps + 1);
}

void orc_revolve_init(orc_revolve *r, int steps, int snaps) {
    memset(r, 0, sizeof(*r));
    r->check = -1; r->capo = 0; r->fine = steps; r->snaps = snaps; r->info = 3;
}

int orc_revolve_next(orc_revolve *r) {
    if (r->check < -1 || r->capo > r->fine) return ORC_ERROR;
    if (r->check == -1 && r->capo < r->fine) { r->turn = 0; r->ch[0] = r->capo - 1; }
    const int gap = r->fine - r->capo;
    if (gap == 0) {
        if (r->check == -1 || r->capo == r->ch[0]) { r->check -= 1; return ORC_TERMINATE; }
        r->capo = r->ch[r->check];
        r->oldfine = r->fine;
        return ORC_RESTORE;
    }
    if (gap == 1) {
        r->fine -= 1;
        if (r->check >= 0 && r->ch[r->check] == r->capo) r->check -= 1;
        r->oldfine = r->fine;
        if (r->turn == 0) { r->turn = 1; return ORC_FIRSTURN; }
        return ORC_YOUTURN;
    }
    if (r->check == -1 || r->ch[r->check] != r->capo) {
        r->check += 1;
        if (r->check >= 64) { r->info = 10; return ORC_ERROR; }
        if (r->check + 1 > r->snaps) { r->info = 11; return ORC_ERROR; }
        r->ch[r->check] = r->capo;
        if (r->check == 0) {
            r->oldsnaps = r->snaps;
            if (r->snaps > 64) { r->info = 14; return ORC_ERROR; }
            if (r->info > 0 && orc_numforw(r->fine - r->capo, r->snaps) == -1) { r->info = 12; return ORC_ERROR; }
        }
        r->oldfine = r->fine;
        return ORC_TAKESHOT;
    }
    if (r->oldfine < r->fine && r->snaps == r->check + 1) { r->info = 13; return ORC_ERROR; }
    const int oldcapo = r->capo;
    const int ds = r->snaps - r->check;
    if (ds < 1) { r->info = 11; return ORC_ERROR; }
    int reps = 0, range = 1;
    while (range < r->fine - r->capo) { reps++; range = range * (reps + ds) / reps; }
    if (reps > 64) { r->info = 15; return ORC_ERROR; }
    if (r->snaps != r->oldsnaps && r->snaps > 64) { r->info = 14; return ORC_ERROR; }
    r->reps = reps; r->range = range;
    const int b1 = range * reps / (ds + reps);
    const int b2 = (ds > 1) ? b1 * ds / (ds + reps - 1) : 1;
    const int b3 = (ds == 1) ? 0 : ((ds > 2) ? b2 * (ds - 1) / (ds + reps - 2) : 1);
    const int b4 = b2 * (reps - 1) / ds;
    const int b5 = (ds < 3) ? 0 : ((ds > 3) ? b3 * (ds - 2) / reps : 1);
    if (r->fine - r->capo <= b1 + b3) r->capo += b4;
    else if (r->fine - r->capo >= range - b5) r->capo += b1;
    else r->capo = r->fine - b2 - b3;
    if (r->capo == oldcapo) r->capo = oldcapo + 1;
    r->oldfine = r->fine;
    return ORC_ADVANCE;
}

int orc_revolve_trace(int steps, int snaps, int *out, int cap) {
    orc_revolve r;
    orc_revolve_init(&r, steps, snaps);
    int n = 0;
    for (;;) {
        int a = orc_revolve_next(&r);
        if (n >= cap) return -1;
        out[3 * n] = a; out[3 * n + 1] = r.capo; out[3 * n + 2] = r.check;
        n++;
        if (a == ORC_TERMINATE || a == ORC_ERROR) break;
    }
    return n;
}

/* ======================================================================== */
/* One time step, literal transcription of the reference kernels.            */
/* ======================================================================== */

typedef struct {
    const orc_shot *s;
    int nxx, nzz, N, nx, nz;
    fft2 f;
    double *i_ax, *i_bx, *i_az, *i_bz, *h_ax, *h_bx, *h_az, *h_bz;
    double *kxsmr, *kxscr, *kzsmr, *kzscr, *kxsmi, *kxsci, *kzsmi, *kzsci;
    double *k2d1, *k2d2, *k2d3, *k2da;
    cplx *dis0, *dis1, *dis2, *dis3, *dis4;
    double *total;
} ctx_t;

/* state layout: 8 consecutive fields */
enum { F_P = 0, F_VX, F_VZ, F_FIPX, F_FIPZ, F_FIVXX, F_FIVZZ, F_AUX, NFIELD };

static int is_visco(int kind) { return kind == ORC_VAPS || kind == ORC_QRTM; }

static void ctx_init(ctx_t *c, const orc_shot *s) {
    memset(c, 0, sizeof(*c));
    c->s = s;
    c->nxx = s->nxx; c->nzz = s->nzz; c->N = s->nxx * s->nzz;
    c->nx = s->nxx - 2 * s->pml; c->nz = s->nzz - 2 * s->pml;
    c->f.nxx = s->nxx; c->f.nzz = s->nzz;
    c->f.px = fft_plan(s->nxx); c->f.pz = fft_plan(s->nzz);
    const int nxx = s->nxx, nzz = s->nzz;
    c->i_ax = malloc(8 * nxx); c->i_bx = malloc(8 * nxx); c->h_ax = malloc(8 * nxx); c->h_bx = malloc(8 * nxx);
    c->i_az = malloc(8 * nzz); c->i_bz = malloc(8 * nzz); c->h_az = malloc(8 * nzz); c->h_bz = malloc(8 * nzz);
    orc_pml_coeffs(s->pml, s->fd, nxx, nzz, s->dx, s->dz, s->dt, c->i_ax, c->i_bx, c->i_az, c->i_bz,
                   c->h_ax, c->h_bx, c->h_az, c->h_bz);
    c->kxsmr = malloc(8 * nxx); c->kxscr = malloc(8 * nxx); c->kxsmi = malloc(8 * nxx); c->kxsci = malloc(8 * nxx);
    c->kzsmr = malloc(8 * nzz); c->kzscr = malloc(8 * nzz); c->kzsmi = malloc(8 * nzz); c->kzsci = malloc(8 * nzz);
    orc_shift_tables(nxx, nzz, s->dx, s->dz, c->kxsmr, c->kxscr, c->kzsmr, c->kzscr,
                     c->kxsmi, c->kxsci, c->kzsmi, c->kzsci);
    const size_t N = (size_t)c->N;
    c->k2d1 = malloc(8 * N); c->k2d2 = malloc(8 * N); c->k2d3 = malloc(8 * N); c->k2da = malloc(8 * N);
    orc_k2d(nxx, nzz, s->dx, s->dz, c->k2d1, c->k2d2, c->k2d3, c->k2da);
    c->dis0 = malloc(sizeof(cplx) * N); c->dis1 = malloc(sizeof(cplx) * N);
    c->dis2 = malloc(sizeof(cplx) * N); c->dis3 = malloc(sizeof(cplx) * N);
    c->dis4 = malloc(sizeof(cplx) * N);
    c->total = malloc(8 * N);
}

static void ctx_free(ctx_t *c) {
    fft_free(c->f.px); fft_free(c->f.pz);
    free(c->i_ax); free(c->i_bx); free(c->i_az); free(c->i_bz);
    free(c->h_ax); free(c->h_bx); free(c->h_az); free(c->h_bz);
    free(c->kxsmr); free(c->kxscr); free(c->kzsmr); free(c->kzscr);
    free(c->kxsmi); free(c->kxsci); free(c->kzsmi); free(c->kzsci);
    free(c->k2d1); free(c->k2d2); free(c->k2d3); free(c->k2da);
    free(c->dis0); free(c->dis1); free(c->dis2); free(c->dis3); free(c->dis4);
    free(c->total);
}

/* Multiply by the derivative-with-shift symbol the way shift_vxz_kernel /
 * shift_pxz_kernel do (sgpstd-qmodeling/acps4.cu:1047-1108, 1210-1271):
 * lower half (i < n/2+1): out = (-a*y - b*x, a*x - b*y); upper half
 * (i > n/2): out = (a*y + b*x, -a*x + b*y); then divide by N. */
static inline cplx shift_mul(cplx in, double a, double b, int i, int n, double N) {
    double x = creal(in), y = cimag(in), re, im;
    if (i < n / 2 + 1) { re = -a * y - b * x; im = a * x - b * y; }
    else { re = a * y + b * x; im = -a * x + b * y; }
    return (re / N) + I * (im / N);
}

/* Stabilised loss symbol, sgpstd-qrtm/acsglw.cu:1895-1924 (multt_kernel),
 * eta scaled by 1e-6. */
static inline double stab_symbol(double k, double eta, double tao, double dt, int nt) {
    const double tt = nt * dt;
    return k - 2.0 * eta * k * (1.0 + tao * dt * k) / 1000000.0 /
                   (exp(-tao * tt * k) + eta * exp(tao * dt * k) / 1000000.0);
}

/* Velocity-divergence stage shared by all four programs:
 * fuzhi_kernel, 2 forward FFTs, shift_vxz_kernel, 2 inverse FFTs,
 * update_vxx_vzz, sumpxpz (sgpstd-qmodeling/acps4.cu:517-552).
 * Leaves div (complex) in dis0. */
static void stage_div(ctx_t *c, double *st) {
    const int nxx = c->nxx, nzz = c->nzz;
    const double Nd = (double)c->N;
    double *vx = st + (size_t)F_VX * c->N, *vz = st + (size_t)F_VZ * c->N;
    double *fivxx = st + (size_t)F_FIVXX * c->N, *fivzz = st + (size_t)F_FIVZZ * c->N;
    for (int i = 0; i < c->N; i++) { c->dis0[i] = vx[i]; c->dis1[i] = vz[i]; }
    fft2_exec(&c->f, c->dis0, -1);
    fft2_exec(&c->f, c->dis1, -1);
#pragma omp parallel for
    for (int ix = 0; ix < nxx; ix++)
        for (int iz = 0; iz < nzz; iz++) {
            size_t a = (size_t)ix * nzz + iz;
            c->dis2[a] = shift_mul(c->dis0[a], c->kxsmr[ix], c->kxsmi[ix], ix, nxx, Nd);
            c->dis3[a] = shift_mul(c->dis1[a], c->kzscr[iz], c->kzsci[iz], iz, nzz, Nd);
        }
    fft2_exec(&c->f, c->dis2, +1);
    fft2_exec(&c->f, c->dis3, +1);
#pragma omp parallel for
    for (int ix = 0; ix < nxx; ix++)
        for (int iz = 0; iz < nzz; iz++) {
            size_t a = (size_t)ix * nzz + iz;
            double sx = creal(c->dis2[a]);
            fivxx[a] = c->i_bx[ix] * fivxx[a] + c->i_ax[ix] * sx;
            c->dis2[a] = (creal(c->dis2[a]) + fivxx[a]) + I * cimag(c->dis2[a]);
            double sz = creal(c->dis3[a]);
            fivzz[a] = c->i_bz[iz] * fivzz[a] + c->i_az[iz] * sz;
            c->dis3[a] = (creal(c->dis3[a]) + fivzz[a]) + I * cimag(c->dis3[a]);
            c->dis0[a] = c->dis2[a] + c->dis3[a];
        }
}

/* Pressure-gradient stage and velocity update: fuzhi_kernel_p, FFT,
 * shift_pxz_kernel, 2 inverse FFTs, vx_cal_kernel, vz_cal_kernel
 * (sgpstd-qmodeling/acps4.cu:571-607); for visco/Q the aux field is
 * refreshed from the same spectrum (acsglw.cu:623-628, qrtm acsglw.cu:611-617). */
static void stage_grad(ctx_t *c, double *st, int t, double eta, int aux_nt) {
    const int nxx = c->nxx, nzz = c->nzz, kind = c->s->kind;
    const double Nd = (double)c->N, dt = c->s->dt;
    double *p = st + (size_t)F_P * c->N, *vx = st + (size_t)F_VX * c->N, *vz = st + (size_t)F_VZ * c->N;
    double *fipx = st + (size_t)F_FIPX * c->N, *fipz = st + (size_t)F_FIPZ * c->N;
    double *aux = st + (size_t)F_AUX * c->N;
    (void)t;
    for (int i = 0; i < c->N; i++) c->dis0[i] = p[i];
    fft2_exec(&c->f, c->dis0, -1);
#pragma omp parallel for
    for (int ix = 0; ix < nxx; ix++)
        for (int iz = 0; iz < nzz; iz++) {
            size_t a = (size_t)ix * nzz + iz;
            c->dis1[a] = shift_mul(c->dis0[a], c->kxscr[ix], c->kxsci[ix], ix, nxx, Nd);
            c->dis2[a] = shift_mul(c->dis0[a], c->kzsmr[iz], c->kzsmi[iz], iz, nzz, Nd);
        }
    fft2_exec(&c->f, c->dis1, +1);
    fft2_exec(&c->f, c->dis2, +1);
    if (is_visco(kind)) {
#pragma omp parallel for
        for (int i = 0; i < c->N; i++) {
            double sym = (kind == ORC_VAPS) ? c->k2da[i]
                                            : stab_symbol(c->k2da[i], eta, c->s->taoc, dt, aux_nt);
            c->dis3[i] = c->dis0[i] * sym / Nd;
        }
        fft2_exec(&c->f, c->dis3, +1);
        for (int i = 0; i < c->N; i++) aux[i] = creal(c->dis3[i]);
    }
#pragma omp parallel for
    for (int ix = 0; ix < nxx; ix++)
        for (int iz = 0; iz < nzz; iz++) {
            size_t a = (size_t)ix * nzz + iz;
            double sx = creal(c->dis1[a]);
            fipx[a] = c->h_bx[ix] * fipx[a] + c->h_ax[ix] * sx;
            vx[a] = vx[a] + dt * c->s->bbx[a] * (sx + fipx[a]);
            double sz = creal(c->dis2[a]);
            fipz[a] = c->h_bz[iz] * fipz[a] + c->h_az[iz] * sz;
            vz[a] = vz[a] + dt * c->s->bbz[a] * (sz + fipz[a]);
        }
}

/* Pressure update.  side 0 = source wavefield (addsa_kernel), side 1 =
 * receiver wavefield (addsa_b_kernel with the Dirichlet overwrite at the
 * receivers from obs row `row`).
 *   aps/artm : p += rho vp^2 dt (div - (vp dt)^2/12 L)        acps4.cu:1488
 *   vaps     : p += rho vp^2 dt lam (total - dt tau D/2) - dt tau aux   acsglw.cu:1527
 *   qrtm     : p += rho vp^2 dt lam (total + dt tau D/2) + dt tau aux   qrtm acsglw.cu:1796
 */
static void stage_p(ctx_t *c, double *st, int t, int side, const double *obs, int row,
                    double *ssg, int restart, const int *rcell, int nrcell) {
    const orc_shot *s = c->s;
    const int nxx = c->nxx, nzz = c->nzz, kind = s->kind;
    const double Nd = (double)c->N, dt = s->dt;
    double *p = st + (size_t)F_P * c->N, *aux = st + (size_t)F_AUX * c->N;
    if (!is_visco(kind)) {
        /* dis1 = F(div); dis2 = dis1 * k2d1 / N; dis2 = F^-1 dis2 */
        memcpy(c->dis1, c->dis0, sizeof(cplx) * (size_t)c->N);
        fft2_exec(&c->f, c->dis1, -1);
        for (int i = 0; i < c->N; i++) c->dis2[i] = c->dis1[i] * c->k2d1[i] / Nd;
        fft2_exec(&c->f, c->dis2, +1);
#pragma omp parallel for
        for (int i = 0; i < c->N; i++) {
            double vp = s->vp[i];
            p[i] = p[i] + s->rho[i] * vp * vp * dt *
                              (creal(c->dis0[i]) - 1.0 / 12.0 * vp * dt * vp * dt * creal(c->dis2[i]));
        }
    } else if (s->lr_row > 0) {
        /* low-rank form: psc = sum_a U[x][a] sum_b A[a][b] Re F^-1[Vt_b F div] / N
         * (multv_kernel / sumlw_kernel / sumlw2_kernel, acsglw.cu:1375-1497, with
         * the sums in double), then p += rho vp^2 dt psc -/+ dt tau aux (the
         * dormant addsa_b_kernel, acsglw.cu:1542-1571, for the pressure term) */
        const int row = s->lr_row, col = s->lr_col;
        memcpy(c->dis1, c->dis0, sizeof(cplx) * (size_t)c->N);
        fft2_exec(&c->f, c->dis1, -1);
        double *pst = calloc((size_t)col * c->N, 8);
        for (int b = 0; b < row; b++) {
            const double *vt = s->lr_Vt + (size_t)b * c->N;
            for (int i = 0; i < c->N; i++) c->dis2[i] = c->dis1[i] * vt[i] / Nd;
            fft2_exec(&c->f, c->dis2, +1);
#pragma omp parallel for
            for (int i = 0; i < c->N; i++)
                for (int a = 0; a < col; a++) pst[(size_t)a * c->N + i] += s->lr_A[a * row + b] * creal(c->dis2[i]);
        }
        const double sg = (kind == ORC_VAPS) ? -1.0 : +1.0;
#pragma omp parallel for
        for (int i = 0; i < c->N; i++) {
            double psc = 0.0;
            for (int a = 0; a < col; a++) psc += s->lr_U[(size_t)i * col + a] * pst[(size_t)a * c->N + i];
            const double vp = s->vp[i];
            p[i] = p[i] + s->rho[i] * vp * vp * dt * psc + sg * dt * s->tao[i] * aux[i];
        }
        free(pst);
    } else {
        memcpy(c->dis1, c->dis0, sizeof(cplx) * (size_t)c->N);
        fft2_exec(&c->f, c->dis1, -1);
        for (int i = 0; i < c->N; i++) {
            c->dis2[i] = c->dis1[i] * c->k2d2[i] / Nd;
            c->dis3[i] = c->dis1[i] * c->k2d1[i] / Nd;
            c->dis4[i] = c->dis1[i] * c->k2d3[i] / Nd;
        }
        fft2_exec(&c->f, c->dis2, +1);
        fft2_exec(&c->f, c->dis3, +1);
        fft2_exec(&c->f, c->dis4, +1);
        /* sum_total (acsglw.cu:1213-1245) */
        for (int i = 0; i < c->N; i++) {
            double g = s->gam[i], w = s->vwd[i], vp = s->vp[i];
            double y1 = 1.0 - 32.0 * g, y2 = 32.0 * g * w, y3 = 1.0 - 64.0 * g, y4 = 64.0 * g * w;
            c->total[i] = y1 * creal(c->dis0[i]) + y2 * creal(c->dis2[i]) -
                          1.0 / 12.0 * dt * dt * vp * vp * s->lam[i] *
                              (y3 * creal(c->dis3[i]) + y4 * creal(c->dis4[i]));
        }
        for (int i = 0; i < c->N; i++) c->dis1[i] = c->total[i];
        fft2_exec(&c->f, c->dis1, -1);
        for (int i = 0; i < c->N; i++) c->dis0[i] = c->dis1[i] * c->k2da[i] / Nd;
        fft2_exec(&c->f, c->dis0, +1);
        const double sg = (kind == ORC_VAPS) ? -1.0 : +1.0;
#pragma omp parallel for
        for (int i = 0; i < c->N; i++) {
            double vp = s->vp[i], tao = s->tao[i];
            p[i] = p[i] + s->rho[i] * vp * vp * dt * s->lam[i] *
                              (c->total[i] + sg * 0.5 * dt * tao * creal(c->dis0[i])) +
                   sg * dt * tao * aux[i];
        }
    }
    if (side == 0) {
        p[(size_t)s->xsg * nzz + s->zsg] += s->rik[t] * dt * 1000.0;
        if (ssg && restart == 0) {
            const int pml = s->pml, nz = c->nz;
            for (int ix = pml; ix < nxx - pml; ix++)
                for (int iz = pml; iz < nzz - pml; iz++) {
                    double v = p[(size_t)ix * nzz + iz];
                    ssg[(size_t)(ix - pml) * nz + (iz - pml)] += v * v;
                }
        }
    } else {
        for (int q = 0; q < nrcell; q++) {
            int cell = rcell[2 * q], ir = rcell[2 * q + 1];
            p[cell] = obs[(size_t)row * s->nr + ir];
        }
    }
}

static void step_source(ctx_t *c, double *st, int t, double *ssg, int restart) {
    stage_div(c, st);
    stage_p(c, st, t, 0, NULL, 0, ssg, restart, NULL, 0);
}

/* ======================================================================== */
/* Drivers                                                                   */
/* ======================================================================== */

/* Source-side steps.  For artm / qrtm these are the steps of the first forward
 * sweep (the advance branch, sgpstd-qrtm/acsglw.cu:508-512), the Q-RTM aux filter at time index t
 * with eta = etas; illumination is not accumulated here. */
int orc_model_steps(const orc_shot *s, double *st, int t0, int nsteps, double *gather) {
    if (s->kind < ORC_APS || s->kind > ORC_QRTM) return -1;
    const double eta = (s->kind == ORC_QRTM) ? s->etas : 0.0;
    ctx_t c;
    ctx_init(&c, s);
    for (int t = t0; t < t0 + nsteps; t++) {
        step_source(&c, st, t, NULL, 1);
        if (gather) {
            const double *p = st + (size_t)F_P * c.N;
            for (int i = 0; i < s->nr; i++)
                gather[(size_t)(t - t0) * s->nr + i] = p[(size_t)s->gxg[i] * s->nzz + s->gzg[i]];
        }
        stage_grad(&c, st, t, eta, t);
    }
    ctx_free(&c);
    return 0;
}

int orc_model_shot(const orc_shot *s, double *gather, double *state) {
    const size_t N = (size_t)s->nxx * s->nzz;
    double *st = calloc(NFIELD * N, sizeof(double));
    int rc = orc_model_steps(s, st, 0, s->nt, gather);
    if (state) memcpy(state, st, sizeof(double) * NFIELD * N);
    free(st);
    return rc;
}

/* Receiver cells: the reference marks flagrec/rindex per grid cell, so when two
 * receivers share a cell the higher index wins (acsglw.cu:387-403). */
static int build_rcells(const orc_shot *s, int *rc) {
    int n = 0;
    for (int i = 0; i < s->nr; i++) {
        int cell = s->gxg[i] * s->nzz + s->gzg[i], found = -1;
        for (int q = 0; q < n; q++) if (rc[2 * q] == cell) { found = q; break; }
        if (found >= 0) rc[2 * found + 1] = i;
        else { rc[2 * n] = cell; rc[2 * n + 1] = i; n++; }
    }
    return n;
}

/* Revolve-driven RTM, sgpstd-qrtm/acsglw.cu:470-1039 (qrtm) and
 * sgpstd-qrtm/acps4.cu:449-905 (artm). */
int orc_rtm_shot(const orc_shot *s, const double *obs, double *img, double *ssg) {
    if (s->kind != ORC_ARTM && s->kind != ORC_QRTM) return -1;
    ctx_t c;
    ctx_init(&c, s);
    const size_t N = (size_t)c.N;
    const int nx = c.nx, nz = c.nz, nzz = s->nzz, pml = s->pml, tmax = s->nt;
    double *src = calloc(NFIELD * N, 8), *rcv = calloc(NFIELD * N, 8);
    double *store = calloc((size_t)s->snaps * NFIELD * N, 8);
    int *rcell = malloc(sizeof(int) * 2 * (size_t)(s->nr > 0 ? s->nr : 1));
    int nrcell = build_rcells(s, rcell);
    memset(img, 0, sizeof(double) * (size_t)nx * nz);
    memset(ssg, 0, sizeof(double) * (size_t)nx * nz);
    orc_revolve r;
    orc_revolve_init(&r, tmax, s->snaps);
    int ts = 0, restart = 0, fwd = 0, act;
    do {
        act = orc_revolve_next(&r);
        if (act == ORC_TAKESHOT && r.info > 1) {
            memcpy(store + (size_t)r.check * NFIELD * N, src, sizeof(double) * NFIELD * N);
            if (r.capo == 0) /* addsource into checkpoint p (acsglw.cu:493-500, 1999-2016) */
                store[(size_t)r.check * NFIELD * N + (size_t)s->xsg * nzz + s->zsg] += s->rik[0] * 1000.0 * s->dt;
        } else if (act == ORC_ADVANCE && r.info > 2) {
            for (int t = ts; t <= r.capo; t++) {
                step_source(&c, src, t, ssg, restart);
                stage_grad(&c, src, t, s->etas, t);
                fwd++;
            }
            ts = r.capo + 1;
        } else if ((act == ORC_FIRSTURN || act == ORC_YOUTURN) && r.info > 2) {
            int row, aux_nt;
            if (act == ORC_FIRSTURN) { restart = 1; row = tmax - 1; aux_nt = tmax - 1; }
            else { row = r.capo; aux_nt = r.capo; }
            stage_div(&c, rcv);
            stage_p(&c, rcv, row, 1, obs, row, NULL, 1, rcell, nrcell);
            stage_grad(&c, rcv, row, s->etar, aux_nt);
            const double *ps = src + (size_t)F_P * N, *pr = rcv + (size_t)F_P * N;
            for (int ix = pml; ix < s->nxx - pml; ix++)
                for (int iz = pml; iz < nzz - pml; iz++) {
                    size_t a = (size_t)ix * nzz + iz;
                    img[(size_t)(ix - pml) * nz + (iz - pml)] += ps[a] * pr[a];
                }
        } else if (act == ORC_RESTORE && r.info > 2) {
            memcpy(src, store + (size_t)r.check * NFIELD * N, sizeof(double) * NFIELD * N);
            ts = r.capo + 1;
        } else if (act == ORC_ERROR) {
            fwd = -1;
            break;
        }
    } while (act != ORC_TERMINATE && act != ORC_ERROR);
    free(src); free(rcv); free(store); free(rcell);
    ctx_free(&c);
    return fwd;
}

/* In-bounds 5-point Laplacian with the border set to zero
 * (sgpstd-qrtm/acsglw.cu:1872-1893 minus its out-of-range writes). */
void orc_filter_image(int nx, int nz, double dx, double dz, const double *img, double *imgf) {
    for (int ix = 0; ix < nx; ix++)
        for (int iz = 0; iz < nz; iz++) {
            size_t a = (size_t)ix * nz + iz;
            if (ix == 0 || iz == 0 || ix == nx - 1 || iz == nz - 1) { imgf[a] = 0.0; continue; }
            imgf[a] = (img[a + 1] + img[a - 1] - 2.0 * img[a]) / dz / dz +
                      (img[a + nz] + img[a - nz] - 2.0 * img[a]) / dx / dx;
        }
}
