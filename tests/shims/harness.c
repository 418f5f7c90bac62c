/*
 * harness.c -- stands in for a reference program's main to drive one
 * acforward shim (tests only).  Build with -DPROG_APS, -DPROG_VAPS, -DPROG_ARTM
 * or -DPROG_QRTM and link the matching shim object, libqpstd and the oracle's
 * restated host helpers.  Run from <dir>/run: it reads <dir>/in/params.txt
 * (tmax dt nshot nrmx nx nz nxx nzz pml dx dz sroffmx disx nxt nzt fd snapnum
 * fobs v0 etas etar flagout), the float32 files in/rik.bin, in/shots.bin
 * (nshot x [shotid, xs, zs]), in/tracenum.bin, the full models in/<name>.bin,
 * and the geometry in/gxp<id>.bin / in/gzp<id>.bin; RTM reads observed data
 * from in/obs<id>_<nr>.bin and writes out/img.bin, out/ssg.bin.  Modeling
 * writes ../obsdata/ as the reference's programs do.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct MultiGPU {
    int *shotid;
    float *sxp;
    float *szp;
};

#if defined(PROG_APS)
void acforward(int, int, int, float, float *, int, int, int, struct MultiGPU *, float *, float *, int, int, int, int,
               int, int, float, float, float, float, float *, float *, float *, float *, int, int, int *, int,
               float *, float *, float *, float *, float *, float *, float *, float *, float *, float *, float *,
               float *, float *, float *, float *, float *, float *, char *, char *);
#elif defined(PROG_VAPS)
void acforward(int, int, int, float, float *, int, int, int, struct MultiGPU *, float *, float *, int, int, int, int,
               int, int, float, float, float *, float *, float *, float *, float, float, float *, float *, float *,
               float *, float *, float *, float *, float *, int, int, int *, int, float *, float *, float *,
               float *, float *, float *, float *, float *, float *, float *, float *, float *, float *, float *,
               float *, float *, char *, char *);
#elif defined(PROG_ARTM)
void acforward(int, int, int, float, float *, int, int, int, struct MultiGPU *, float *, float *, int, int, int, int,
               int, int, float, float, float *, float *, float *, float *, float, float, float *, float *, float *,
               float *, int, int, int *, float *, float *, float *, float *, float *, float *, float *, float *,
               float *, float *, float *, float *, float *, float *, float *, float *, float *, float *, float,
               float, char *, char *, char *);
#elif defined(PROG_QRTM)
void acforward(int, int, int, float, float *, int, int, int, struct MultiGPU *, float *, float *, int, int, int, int,
               int, int, float, float, float *, float *, float *, float *, float, float, float *, float *, float *,
               float *, float *, float *, float *, float *, int, int, int *, float *, float *, float *, float *,
               float *, float *, float *, float *, float *, float *, float *, float *, float *, float *, float *,
               float *, float *, float *, float, float, float, float, char *, char *, char *);
#endif

static void *load(const char *dir, const char *name, size_t n, size_t size) {
    char path[512];
    snprintf(path, sizeof path, "%s/in/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(2);
    }
    void *p = calloc(n ? n : 1, size);
    if (fread(p, size, n, f) != n) {
        fprintf(stderr, "short file %s\n", path);
        exit(2);
    }
    fclose(f);
    return p;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const char *dir = argv[1];
    char path[512];
    snprintf(path, sizeof path, "%s/in/params.txt", dir);
    FILE *pf = fopen(path, "r");
    if (!pf) return 2;
    int tmax, nshot, nrmx, nx, nz, nxx, nzz, pml, nxt, nzt, snapnum, flagout;
    float dt, dx, dz, sroffmx, disx, fd, fobs, v0, etas, etar;
    if (fscanf(pf, "%d %f %d %d %d %d %d %d %d %f %f %f %f %d %d %f %d %f %f %f %f %d", &tmax, &dt, &nshot, &nrmx,
               &nx, &nz, &nxx, &nzz, &pml, &dx, &dz, &sroffmx, &disx, &nxt, &nzt, &fd, &snapnum, &fobs, &v0, &etas,
               &etar, &flagout) != 22)
        return 2;
    fclose(pf);
    float *rik = load(dir, "rik.bin", tmax, sizeof(float));
    float *shots = load(dir, "shots.bin", 3 * (size_t)nshot, sizeof(float));
    int *tracenum = load(dir, "tracenum.bin", 64, sizeof(int));
    const size_t NT = (size_t)nxt * nzt;
    float *vpt = load(dir, "vp.bin", NT, 4), *rhot = load(dir, "rho.bin", NT, 4);
    float *bbxt = load(dir, "bbx.bin", NT, 4), *bbzt = load(dir, "bbz.bin", NT, 4);
#if defined(PROG_VAPS) || defined(PROG_QRTM)
    float *gamt = load(dir, "gam.bin", NT, 4), *lamt = load(dir, "lam.bin", NT, 4);
    float *vwdt = load(dir, "vwd.bin", NT, 4), *taot = load(dir, "tao.bin", NT, 4);
#endif
    struct MultiGPU sg;
    sg.shotid = calloc(nshot, sizeof(int));
    sg.sxp = calloc(nshot, sizeof(float));
    sg.szp = calloc(nshot, sizeof(float));
    for (int i = 0; i < nshot; i++) {
        sg.shotid[i] = (int)shots[3 * i];
        sg.sxp[i] = shots[3 * i + 1];
        sg.szp[i] = shots[3 * i + 2];
    }
    float *gxp = calloc(nrmx, sizeof(float)), *gzp = calloc(nrmx, sizeof(float));
    /* coefficient tables: the shim reads only the interior CPML decay */
    float *tx[8], *tz[8], *k2[4];
    for (int k = 0; k < 8; k++) {
        tx[k] = calloc(nxx, sizeof(float));
        tz[k] = calloc(nzz, sizeof(float));
    }
    for (int k = 0; k < 4; k++) k2[k] = calloc((size_t)nxx * nzz, sizeof(float));
    for (int i = 0; i < nxx; i++) tx[1][i] = (float)exp(-(double)dt * 3.1415926 * fd);
    char f4[40], f5[40], recname[60];
    snprintf(f4, sizeof f4, "%s/in/gxp", dir);
    snprintf(f5, sizeof f5, "%s/in/gzp", dir);
    snprintf(recname, sizeof recname, "%s/in/obs", dir);
    (void)snapnum, (void)fobs, (void)v0, (void)etas, (void)etar, (void)recname, (void)flagout;
#if defined(PROG_APS)
    acforward(snapnum, 1, tmax, dt, rik, 0, 1, nshot, &sg, gxp, gzp, nrmx, nx, nz, nxx, nzz, pml, dx, dz, sroffmx,
              disx, vpt, rhot, bbxt, bbzt, nxt, nzt, tracenum, flagout, k2[0], tx[0], tx[1], tz[0], tz[1], tx[2],
              tx[3], tz[2], tz[3], tx[4], tx[5], tz[4], tz[5], tx[6], tx[7], tz[6], tz[7], f4, f5);
#elif defined(PROG_VAPS)
    acforward(snapnum, 1, tmax, dt, rik, 0, 1, nshot, &sg, gxp, gzp, nrmx, nx, nz, nxx, nzz, pml, dx, dz, k2[0],
              k2[1], k2[2], k2[3], sroffmx, disx, vpt, vwdt, taot, lamt, gamt, rhot, bbxt, bbzt, nxt, nzt,
              tracenum, flagout, tx[0], tx[1], tz[0], tz[1], tx[2], tx[3], tz[2], tz[3], tx[4], tx[5], tz[4],
              tz[5], tx[6], tx[7], tz[6], tz[7], f4, f5);
#else
    float *img_sp = calloc(NT, sizeof(float)), *ssg_sp = calloc(NT, sizeof(float));
#if defined(PROG_ARTM)
    acforward(snapnum, 1, tmax, dt, rik, 0, 1, nshot, &sg, gxp, gzp, nrmx, nx, nz, nxx, nzz, pml, dx, dz, k2[0],
              k2[1], k2[2], k2[3], sroffmx, disx, vpt, rhot, bbxt, bbzt, nxt, nzt, tracenum, tx[0], tx[1], tz[0],
              tz[1], tx[2], tx[3], tz[2], tz[3], tx[4], tx[5], tz[4], tz[5], tx[6], tx[7], tz[6], tz[7], img_sp,
              ssg_sp, fobs, v0, f4, f5, recname);
#else
    acforward(snapnum, 1, tmax, dt, rik, 0, 1, nshot, &sg, gxp, gzp, nrmx, nx, nz, nxx, nzz, pml, dx, dz, k2[0],
              k2[1], k2[2], k2[3], sroffmx, disx, vpt, vwdt, taot, lamt, gamt, rhot, bbxt, bbzt, nxt, nzt,
              tracenum, tx[0], tx[1], tz[0], tz[1], tx[2], tx[3], tz[2], tz[3], tx[4], tx[5], tz[4], tz[5], tx[6],
              tx[7], tz[6], tz[7], img_sp, ssg_sp, fobs, v0, etas, etar, f4, f5, recname);
#endif
    snprintf(path, sizeof path, "%s/out/img.bin", dir);
    FILE *fo = fopen(path, "wb");
    if (!fo) return 3;
    fwrite(img_sp, sizeof(float), NT, fo);
    fclose(fo);
    snprintf(path, sizeof path, "%s/out/ssg.bin", dir);
    fo = fopen(path, "wb");
    if (!fo) return 3;
    fwrite(ssg_sp, sizeof(float), NT, fo);
    fclose(fo);
#endif
    return 0;
}
