// acforward_aps.cpp -- acforward of the aps program (acoustic modeling) with
// the signature of sgpstd-qmodeling/acps4.cu:184-198, on libqpstd.
#include "acforward_common.h"

extern "C" void acforward(int snapnum, int GPU_N, int tmax, float dt, float *rik, int myid, int numprocs, int nshot,
                          struct MultiGPU singpu[], float *gxp, float *gzp, int nrmx, int nx, int nz, int nxx,
                          int nzz, int pml, float dx, float dz, float sroffmx, float disx, float *vpt, float *rhot,
                          float *bbxt, float *bbzt, int nxt, int nzt, int *tracenum, int flagout, float *k2d1,
                          float *i_ax, float *i_bx, float *i_az, float *i_bz, float *h_ax, float *h_bx,
                          float *h_az, float *h_bz, float *kxsmr, float *kxscr, float *kzsmr, float *kzscr,
                          float *kxsmi, float *kxsci, float *kzsmi, float *kzsci, char fname4[40],
                          char fname5[40]) {
    (void)snapnum, (void)numprocs, (void)k2d1;
    (void)kxsmr, (void)kxscr, (void)kzsmr, (void)kzscr, (void)kxsmi, (void)kxsci;
    (void)kzsmi, (void)kzsci;
    if (!qpshim::one_gpu(GPU_N)) return;
    qpshim::Common c{tmax, dt, rik, myid, gxp, gzp, nrmx, nx, nz, nxx, nzz, pml, dx, dz, sroffmx, disx,
                           nxt, nzt, tracenum, i_bx, fname4, fname5};
    qpshim::set_cpml(c, i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz);
    float *models[8] = {vpt, rhot, bbxt, bbzt, nullptr, nullptr, nullptr, nullptr};
    qpshim::model(c, singpu, nshot, models, QPSTD_APS, flagout, "reca", "snapa");
}
