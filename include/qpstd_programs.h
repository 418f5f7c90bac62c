/*
 * qpstd_programs.h -- host-side C ABI of the native programs (libqpstd_host.so).
 *
 * The reference's four programs read a parameter file, generate or read the
 * acquisition geometry and set up the full model on the host before acforward
 * runs the shots.  These entry points expose that host work, in the
 * reference's float arithmetic, for callers that drive libqpstd themselves and
 * for tests; the `qpstd` executable (aps / vaps / artm / qrtm / geometry / sum)
 * is built on the same code.  Programs: 0 aps, 1 vaps, 2 artm, 3 qrtm.
 * All functions return 0 on success and a negative value on failure unless
 * stated otherwise.
 */
#ifndef QPSTD_PROGRAMS_H
#define QPSTD_PROGRAMS_H
#ifdef __cplusplus
extern "C" {
#endif

/* Reads a program's parameter file (replaces input_ac2d_parameters:
 * sgpstd-qmodeling/funca.c:9, func.c:9; sgpstd-qrtm/funca.c:9, func.c:9).
 * The numeric values go to nums in file order (at most maxn), the strings to
 * strs as newline-terminated lines (at most strs_len bytes with the NUL).
 * Returns the number of numeric values, or < 0 (message: qpcli_last_error). */
int qpcli_read_params(int program, const char *path, double *nums, int maxn, char *strs, int strs_len);

/* Writes the split-spread geometry files into dir from a geometry parameter
 * file (replaces geometry/geometry2d.c:7-152, which reads parameters.txt in its
 * working directory). */
int qpcli_write_geometry(const char *params_path, const char *dir);

/* Full-model setup (sgpstd-qrtm/func.c:205 cal_bbx_bbz, :237 rik_cal,
 * :939 transfermodel, :555 get_max_min, :569 check_stability_ps). */
void qpcli_cal_bbx_bbz(int nx, int nz, const float *rho, float *bbx, float *bbz);
void qpcli_rik_cal(int tmax, float dt, float fd, int flag, float *rik);
void qpcli_transfermodel(int n, float fd, float fo, const float *vp, const float *qp, float *gam, float *lam,
                         float *vwd, float *tao);
void qpcli_get_max_min(int n, const float *a, float *vmax, float *vmin);
float qpcli_cfl_number(float vmax, float dt, float dx, float dz);

/* First shot and shot count of process rank among nranks, one GPU each
 * (sgpstd-qmodeling/acousticsgps4.c:254-270 with GPU_N = 1). */
void qpcli_distribute(int shotnum, int nranks, int rank, int *first, int *count);
/* Window width nx from the largest offset (acousticsgps4.c:333-334). */
int qpcli_window_width(float sroffmx, float disx, float dx);

const char *qpcli_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
