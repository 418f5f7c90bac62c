// setup.cpp -- what the programs' mains compute on the full model before the
// shots run.  The arithmetic keeps the reference's types (float storage,
// double intermediates where its C expressions promote), so the values are
// the ones its programs pass to acforward.
#include <cmath>

#include "programs.h"

namespace qpcli {

// The reference's pi constant (sgpstd-qrtm/func.c:6), not M_PI.
static constexpr double kPi = 3.1415926;

// Buoyancies on the staggered half points (sgpstd-qrtm/func.c:205-234):
// harmonic means of neighbouring densities, the last column / row the point's own.
void cal_bbx_bbz(int nx, int nz, const float *rho, float *bbx, float *bbz) {
    for (int i = 0; i < nx; i++) {
        const float *r = rho + (size_t)i * nz;
        float *bx = bbx + (size_t)i * nz, *bz = bbz + (size_t)i * nz;
        for (int j = 0; j < nz; j++) {
            bx[j] = (i + 1 < nx) ? (float)(2.0 / (double)(r[j] + r[j + nz])) : (float)(1.0 / (double)r[j]);
            bz[j] = (j + 1 < nz) ? (float)(2.0 / (double)(r[j] + r[j + 1])) : (float)(1.0 / (double)r[j]);
        }
    }
}

// Source wavelet delayed by t0 = 1/fd: Ricker (flag 2) or the first derivative
// of a Gaussian (sgpstd-qrtm/func.c:237-256).
void rik_cal(int tmax, float dt, float fd, int flag, float *rik) {
    const float t0 = (float)(1.0 / fd);
    for (int i = 0; i < tmax; i++) {
        const float tt = (float)i * dt - t0;
        // pow(u, 2), not u * u: the same libm call as the reference, so the
        // float rounding of a matches it in every case
        if (flag == 2) {
            const float a = (float)std::pow(kPi * fd * tt, 2.0);
            rik[i] = (float)((1.0 - 2.0 * a) * std::exp(-(double)a));
        } else {
            const float a = (float)std::pow(2.0 * kPi * fd * tt, 2.0);
            rik[i] = (float)((double)tt * std::exp(-(double)a));
        }
    }
}

// Constant-Q parameters from Qp (sgpstd-qrtm/func.c:939-956): gamma = 1/(pi Q),
// lambda = (fd/fo)^(2 gamma), vwd = (vp/(2 pi fd))^(1/16), tau = lambda vp / Q.
void transfermodel(int n, float fd, float fo, const float *vp, const float *qp, float *gam, float *lam, float *vwd,
                   float *tao) {
    const float wd = (float)(2.0 * kPi * fd);
    const double ratio = (double)(fd / fo);
    for (int i = 0; i < n; i++) {
        gam[i] = (float)(1.0 / kPi / qp[i]);
        lam[i] = (float)std::pow(ratio, 2.0 * (double)gam[i]);
        vwd[i] = (float)std::pow((double)(vp[i] / wd), 1.0 / 16.0);
        tao[i] = lam[i] * vp[i] / qp[i];
    }
}

// Extremes with the reference's 1e-4 hysteresis (sgpstd-qrtm/func.c:555-567).
void get_max_min(int n, const float *a, float *vmax, float *vmin) {
    float mn = 10000000.0f, mx = -10000000.0f;
    for (int i = 0; i < n; i++) {
        if (a[i] - mn < 1.0e-4) mn = a[i];
        if (a[i] - mx > 1.0e-4) mx = a[i];
    }
    *vmax = mx;
    *vmin = mn;
}

// pi vmax dt / 2 sqrt(1/dx^2 + 1/dz^2) (sgpstd-qrtm/func.c:569-574)
float cfl_number(float vmax, float dt, float dx, float dz) {
    return (float)(kPi * vmax * dt / 2.0 * std::sqrt(1.0 / dx / dx + 1.0 / dz / dz));
}

// The first shotnum % nranks processes take one shot more; shots are
// contiguous per process.
void distribute(int shotnum, int nranks, int rank, int *first, int *count) {
    const int rid = shotnum % nranks, ave = (shotnum - rid) / nranks;
    if (rank < rid) {
        *count = ave + 1;
        *first = rank * (ave + 1);
    } else {
        *count = ave;
        *first = rid * (ave + 1) + (rank - rid) * ave;
    }
}

int window_width(float sroffmx, float disx, float dx) {
    const float simxlen = (float)(2.0 * (double)(sroffmx + disx));
    return (int)((double)(simxlen / dx) + 1.5);
}

}  // namespace qpcli
