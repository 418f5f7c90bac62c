// callbacks.cpp -- the host helpers the reference's acforward calls back into
// (extern "C", sgpstd-qmodeling/acps4.cu:142-180), for the native programs.
// The reference-signature acforward shims call these names; a reference
// program links its own, the native tool links these.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

extern "C" {
void select_part_model(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz, float *vpt,
                       float *vp);
void expand_pml_areas(int nx, int nz, int nxx, int nzz, int pml, float *vp);
void input_geophone_pos(int shotid, int nr, float *gxp, char fname[]);
void projectomodel(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz, float *vpt,
                   float *vp);
void removedirect(int nrmx, int tmax, int nr, float dt, float fd, float xs, float zs, float *gxp, float *gzp,
                  float v0, float *recsim);
float get_max_tao(int nxx, int nzz, float *tao);
}

namespace {

// Model column of window column 0: (int)(mlx/dx) when the window starts inside
// the model, -round(|mlx|/dx) when it starts left of it
// (sgpstd-qrtm/funca.c:655, 692).
int window_origin(float mlx, float dx) {
    return (mlx >= 0.0f) ? (int)(mlx / dx) : -(int)(std::fabs((double)mlx) / dx + 0.5);
}

}  // namespace

// Window columns w = 0..nx-1 of the padded nxx x nzz model take model column
// origin + w, clamped to the model (columns off either edge repeat the edge
// column); rows pml..pml+nzt-1 are written (sgpstd-qrtm/funca.c:643-753).
void select_part_model(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz, float *vpt,
                       float *vp) {
    (void)nz, (void)nxx;
    if (nxt < 1) return;
    const int o = window_origin(mlx, dx);
    for (int w = 0; w < nx; w++) {
        const int c = std::min(std::max(o + w, 0), nxt - 1);
        std::copy(vpt + (size_t)c * nzt, vpt + (size_t)(c + 1) * nzt, vp + (size_t)(w + pml) * nzz + pml);
    }
}

// The CPML frame takes the nearest interior value: top and bottom rows of the
// interior columns first, then whole left and right columns
// (sgpstd-qrtm/funca.c:755-790).
void expand_pml_areas(int nx, int nz, int nxx, int nzz, int pml, float *vp) {
    (void)nx, (void)nz;
    for (int i = pml; i < nxx - pml; i++) {
        float *col = vp + (size_t)i * nzz;
        std::fill(col, col + pml, col[pml]);
        std::fill(col + nzz - pml, col + nzz, col[nzz - pml - 1]);
    }
    const float *left = vp + (size_t)pml * nzz, *right = vp + (size_t)(nxx - pml - 1) * nzz;
    for (int i = 0; i < pml; i++) std::copy(left, left + nzz, vp + (size_t)i * nzz);
    for (int i = nxx - pml; i < nxx; i++) std::copy(right, right + nzz, vp + (size_t)i * nzz);
}

// Receiver coordinates of one shot from "<fname><shotid>.bin"
// (sgpstd-qrtm/funca.c:596-609).  A missing file ends the program, as in the
// reference.
void input_geophone_pos(int shotid, int nr, float *gxp, char fname[]) {
    char path[1024];
    std::snprintf(path, sizeof path, "%s%d.bin", fname, shotid);
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        std::printf("Cannot open receiver positions file %s\n", path);
        std::exit(1);
    }
    if (std::fread(gxp, sizeof(float), (size_t)nr, f) != (size_t)nr)
        std::printf("warning: %s holds fewer than %d positions\n", path, nr);
    std::fclose(f);
}

// The nx x nz window image written back into the model frame: model column
// origin + w takes window column w where both exist (sgpstd-qrtm/funca.c:823-896).
void projectomodel(int pml, float mlx, float dx, int nxt, int nzt, int nx, int nz, int nxx, int nzz, float *vpt,
                   float *vp) {
    (void)pml, (void)nxx, (void)nzz;
    const int o = window_origin(mlx, dx);
    for (int c = std::max(o, 0); c < nxt && c - o < nx; c++)
        std::copy(vp + (size_t)(c - o) * nz, vp + (size_t)(c - o) * nz + nzt, vpt + (size_t)c * nzt);
}

// Each trace is zeroed from the direct arrival (offset / v0) for two periods
// of fd (sgpstd-qrtm/funca.c:898-919); the gather is time-major (nt x nr).
void removedirect(int nrmx, int tmax, int nr, float dt, float fd, float xs, float zs, float *gxp, float *gzp,
                  float v0, float *recsim) {
    (void)nrmx;
    const int width = (int)(2.0 / fd / dt + 0.5);
    for (int i = 0; i < nr; i++) {
        const double ox = (double)(xs - gxp[i]), oz = (double)(zs - gzp[i]);
        const float dis = (float)std::sqrt(std::pow(ox, 2.0) + std::pow(oz, 2.0));
        const int ts = (int)(1.0 * dis / v0 / dt + 0.5);
        const int te = std::min(ts + width, tmax - 1);
        for (int t = ts; t <= te; t++) recsim[(size_t)t * nr + i] = 0.0f;
    }
}

// Largest tau of the window, at least 0 (sgpstd-qrtm/func.c:960-970).
float get_max_tao(int nxx, int nzz, float *tao) {
    float m = 0.0f;
    for (long i = 0; i < (long)nxx * nzz; i++) m = (tao[i] >= m) ? tao[i] : m;
    return m;
}
