/*
 * qpstd_oracle.h -- FP64 CPU oracle for the Constant-Q-PSTD time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke()
 * entry point and bench.py's cpu_baseline leg may call it, the product path
 * (the CUDA library under constant-q-pstd_gb300/) never does.
 *
 * It restates, in double precision, the update equations that the reference
 * executes with cuFFT on the GPU (the reference has no CPU stepping path):
 *   - sgpstd-qmodeling/acps4.cu   (aps:  acoustic staggered-grid PSTD)
 *   - sgpstd-qmodeling/acsglw.cu  (vaps: constant-Q power-expansion form)
 *   - sgpstd-qrtm/acps4.cu        (artm: acoustic RTM with revolve)
 *   - sgpstd-qrtm/acsglw.cu       (qrtm: Q-compensated RTM with revolve)
 * The 2-D transforms are complex-to-complex, unnormalised, with the cuFFT sign
 * convention (forward e^{-i}, inverse e^{+i}); intermediate fields are kept
 * complex exactly where the reference keeps them complex (e.g. sumpxpz adds the
 * imaginary parts of the two derivative fields).
 */
#ifndef QPSTD_ORACLE_H
#define QPSTD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_APS = 0, ORC_VAPS = 1, ORC_ARTM = 2, ORC_QRTM = 3 };

/* ---- 1-D FFT (mixed radix + Bluestein), interleaved re/im, unnormalised ---- */
int orc_fft1d(int n, double *re_im, int sign);

/* ---- one-time coefficient setup, FP64 restatements ---------------------- */
void orc_pml_coeffs(int pml, double fm, int nxx, int nzz, double dx, double dz, double dt,
                    double *i_ax, double *i_bx, double *i_az, double *i_bz,
                    double *h_ax, double *h_bx, double *h_az, double *h_bz);
void orc_shift_tables(int nxx, int nzz, double dx, double dz,
                      double *kxsmr, double *kxscr, double *kzsmr, double *kzscr,
                      double *kxsmi, double *kxsci, double *kzsmi, double *kzsci);
void orc_k2d(int nxx, int nzz, double dx, double dz,
             double *k2d1, double *k2d2, double *k2d3, double *k2da);
void orc_ricker(int nt, double dt, double fd, int flag, double *rik);
void orc_bbx_bbz(int nxx, int nzz, const double *rho, double *bbx, double *bbz);
void orc_transfermodel(int n, double fd, double fo, const double *vp, const double *qp,
                       double *gam, double *lam, double *vwd, double *tao);

/* ---- revolve (binomial checkpointing), re-entrant ------------------------ */
enum { ORC_ADVANCE = 0, ORC_TAKESHOT, ORC_RESTORE, ORC_FIRSTURN, ORC_YOUTURN,
       ORC_TERMINATE, ORC_ERROR };
typedef struct {
    int turn, reps, range, oldsnaps, oldfine;
    int ch[64];
    int check, capo, fine, snaps, info;
} orc_revolve;
void orc_revolve_init(orc_revolve *r, int steps, int snaps);
int orc_revolve_next(orc_revolve *r);
int orc_numforw(int steps, int snaps);
/* Writes up to cap (action, capo, check) triples; returns the count or -1. */
int orc_revolve_trace(int steps, int snaps, int *out, int cap);

/* ---- one shot ------------------------------------------------------------ */
typedef struct {
    int kind;                 /* ORC_APS .. ORC_QRTM */
    int nxx, nzz, pml;        /* padded grid and CPML width */
    double dx, dz, dt, fd;    /* dt in seconds; fd = CPML alpha_max / pi */
    int nt;                   /* time samples */
    const double *vp, *rho, *bbx, *bbz;      /* nxx*nzz, x-major */
    const double *gam, *lam, *vwd, *tao;     /* visco / Q only */
    const double *rik;        /* nt */
    int xsg, zsg;             /* source grid index (padded grid) */
    int nr;
    const int *gxg, *gzg;     /* receiver grid indices (padded grid) */
    double etas, etar;        /* Q-RTM stabilisation (scaled by 1e-6 inside) */
    double taoc;              /* Q-RTM filter tau (max tau over the window) */
    int snaps;                /* RTM checkpoints */
    /* Low-rank form of the constant-Q pressure update (lr_row > 0; vaps / qrtm):
     * p += rho vp^2 dt W{div} -/+ dt tau aux, with W{div} = sum_a U[x][a]
     * sum_b A[a][b] Re F^-1[Vt_b F div] / N, the operator of the reference's
     * dormant kernels (sgpstd-qmodeling/acsglw.cu:1375-1497) fed as its dormant
     * pressure update does (addsa_b_kernel, acsglw.cu:1542-1571). */
    int lr_row, lr_col;
    const double *lr_U;       /* nxx*nzz x lr_col */
    const double *lr_Vt;      /* lr_row x nxx*nzz: the half-grid factors mirrored to the full grid */
    const double *lr_A;       /* lr_col x lr_row */
} orc_shot;

/* Forward modeling (aps / vaps).  gather: nt*nr time-major, p after the
 * p-update of each step.  state (optional, may be NULL): final
 * p,vx,vz,fipx,fipz,fivxx,fivzz,aux, each nxx*nzz. */
int orc_model_shot(const orc_shot *s, double *gather, double *state);

/* Run nsteps steps from a given state (8 fields, in/out) starting at step
 * index t0; used by the per-step parity tests.  gather may be NULL. */
int orc_model_steps(const orc_shot *s, double *state, int t0, int nsteps, double *gather);

/* RTM (artm / qrtm) for one shot.  obs: nt*nr time-major (already muted).
 * img, ssg: nx*nz interior arrays, cross-correlation image before the
 * Laplacian filter and the first-sweep illumination.  Returns the number of
 * forward steps executed (revolve recompute included) or -1. */
int orc_rtm_shot(const orc_shot *s, const double *obs, double *img, double *ssg);

/* 5-point Laplacian of the image with the border zeroed (in-bounds form). */
void orc_filter_image(int nx, int nz, double dx, double dz, const double *img, double *imgf);

#ifdef __cplusplus
}
#endif
#endif
