/*
 * host_helpers.c -- TEST INFRASTRUCTURE ONLY: a C restatement of the host-side
 * helpers the reference's programs link into acforward (its extern "C"
 * callbacks, sgpstd-qmodeling/acps4.cu:142-180).  The shim test harness
 * (tests/shims/) links these in place of the reference's own C files, which
 * cannot travel with the repository.  Each function follows the reference
 * file:line named beside it and is pinned against the reference's compiled
 * functions through tests/golden (make_golden.py).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* sgpstd-qrtm/funca.c:596-609: receiver coordinates of one shot from "<fname><shotid>.bin" */
void input_geophone_pos(int shotid, int nr, float *gxp, char fname[40]) {
    char nname[256];
    snprintf(nname, sizeof nname, "%s%d.bin", fname, shotid);
    FILE *fp = fopen(nname, "rb");
    if (!fp) {
        printf("Cannot open receiver positions file!\n");
        exit(0);
    }
    if (fread(gxp, sizeof(float), (size_t)nr, fp) != (size_t)nr) printf("short receiver positions file\n");
    fclose(fp);
}

/* window column c of the padded model from model column src (or from window column src2) */
static void put_col(float *vp, const float *vpt, int nzt, int nzz, int pml, int wcol, int tcol) {
    for (int j = 0; j < nzt; j++) vp[(size_t)(wcol + pml) * nzz + j + pml] = vpt[(size_t)tcol * nzt + j];
}
static void copy_col(float *vp, int nzz, int pml, int wdst, int wsrc) {
    for (int j = pml; j < nzz - pml; j++) vp[(size_t)(wdst + pml) * nzz + j] = vp[(size_t)(wsrc + pml) * nzz + j];
}

/* sgpstd-qrtm/funca.c:643-753: cut window columns [mlx/dx, mlx/dx+nx) of the
 * nxt x nzt model into the padded nxx x nzz window; columns beyond the model
 * repeat the model's edge column. */
void select_part_model(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz,
                       float *vpt, float *vp) {
    (void)nz;
    (void)nxx;
    if (mlx >= 0.0f) {
        const int f0 = (int)(mlx / dx), f1 = f0 + nx - 1;
        if (f1 < nxt) {
            for (int i = f0; i <= f1; i++) put_col(vp, vpt, nzt, nzz, pml, i - f0, i);
        } else {
            for (int i = f0; i < nxt; i++) put_col(vp, vpt, nzt, nzz, pml, i - f0, i);
            for (int i = nxt; i <= f1; i++) copy_col(vp, nzz, pml, i - f0, nxt - 1 - f0);
        }
    }
    if (mlx < 0.0f) {
        const int f0 = (int)(fabs((double)mlx) / dx + 0.5), f1 = nx - f0;
        if (f1 <= nxt) {
            for (int i = 0; i < f1; i++) put_col(vp, vpt, nzt, nzz, pml, i + f0, i);
            for (int i = 0; i < f0; i++) copy_col(vp, nzz, pml, i, f0);
        } else {
            for (int i = 0; i < nxt; i++) put_col(vp, vpt, nzt, nzz, pml, i + f0, i);
            for (int i = nxt; i < f1; i++) copy_col(vp, nzz, pml, i + f0, nxt - 1 + f0);
            for (int i = 0; i < f0; i++) copy_col(vp, nzz, pml, i, f0);
        }
    }
}

/* sgpstd-qrtm/funca.c:755-790: fill the CPML frame from the nearest interior value */
void expand_pml_areas(int nx, int nz, int nxx, int nzz, int pml, float *vp) {
    (void)nx;
    (void)nz;
    for (int i = pml; i < nxx - pml; i++) {
        for (int j = 0; j < pml; j++) vp[(size_t)i * nzz + j] = vp[(size_t)i * nzz + pml];
        for (int j = nzz - pml; j < nzz; j++) vp[(size_t)i * nzz + j] = vp[(size_t)i * nzz + nzz - pml - 1];
    }
    for (int j = 0; j < nzz; j++) {
        for (int i = 0; i < pml; i++) vp[(size_t)i * nzz + j] = vp[(size_t)pml * nzz + j];
        for (int i = nxx - pml; i < nxx; i++) vp[(size_t)i * nzz + j] = vp[(size_t)(nxx - pml - 1) * nzz + j];
    }
}

/* sgpstd-qrtm/funca.c:823-896: the nx x nz window image placed back into the
 * nxt x nzt model frame (vpt out, vp in); only model columns inside the
 * window are written. */
void projectomodel(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz, float *vpt,
                   float *vp) {
    (void)pml;
    (void)nxx;
    (void)nzz;
    if (mlx >= 0.0f) {
        const int f0 = (int)(mlx / dx), f1 = f0 + nx - 1;
        const int last = (f1 < nxt) ? f1 : nxt - 1;
        for (int i = f0; i <= last; i++)
            for (int j = 0; j < nzt; j++) vpt[(size_t)i * nzt + j] = vp[(size_t)(i - f0) * nz + j];
    } else {
        const int f0 = (int)(fabs((double)mlx) / dx + 0.5), f1 = nx - f0;
        const int cnt = (f1 <= nxt) ? f1 : nxt;
        for (int i = 0; i < cnt; i++)
            for (int j = 0; j < nzt; j++) vpt[(size_t)i * nzt + j] = vp[(size_t)(i + f0) * nz + j];
    }
}

/* sgpstd-qrtm/funca.c:898-919: zero each trace from the direct arrival time
 * (offset / v0) for two periods of fd */
void removedirect(int nrmx, int tmax, int nr, float dt, float fd, float xs, float zs, float *gxp, float *gzp,
                  float v0, float *recobs) {
    (void)nrmx;
    for (int i = 0; i < nr; i++) {
        const float dis = (float)sqrt(pow((double)(xs - gxp[i]), 2.0) + pow((double)(zs - gzp[i]), 2.0));
        const int ts = (int)(1.0 * dis / v0 / dt + 0.5);
        int te = ts + (int)(2.0 / fd / dt + 0.5);
        if (te >= tmax) te = tmax - 1;
        for (int j = ts; j <= te; j++) recobs[(size_t)j * nr + i] = 0.0f;
    }
}

/* sgpstd-qrtm/func.c:960-970 */
float get_max_tao(int nxx, int nzz, float *tao) {
    float mn = 0.0f;
    for (int i = 0; i < nxx * nzz; i++)
        if (tao[i] >= mn) mn = tao[i];
    return mn;
}
