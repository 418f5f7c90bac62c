/*
 * qpstd.h -- C ABI of the GB300 Constant-Q-PSTD time-stepping library.
 *
 * The reference exposes its hot path as one `extern "C" void acforward(...)`
 * per program, ~40 positional scalars and host pointers, no status code:
 *   aps  : sgpstd-qmodeling/acps4.cu:184-198   (called acousticsgps4.c:442)
 *   vaps : sgpstd-qmodeling/acsglw.cu:185-200  (called visacousticsgps4.c:455)
 *   artm : sgpstd-qrtm/acps4.cu:183-197        (called main.c:458)
 *   qrtm : sgpstd-qrtm/acsglw.cu:189-204       (called acrtmain.c:459)
 * Each acforward loops over shots; per shot it windows the model
 * (select_part_model / expand_pml_areas), places the source and receivers,
 * time-steps on the GPU and writes the gather (modeling) or accumulates the
 * image (RTM).  The entry points below are that per-shot body with the
 * windowing already done by the caller, taking plain host pointers and sizes
 * and returning a status code; qpstd_acforward_* further down restore the
 * whole-program signatures.
 *
 * Layout conventions (as in the reference): every 2-D array is x-major,
 * point (ix,iz) at ix*nzz+iz; gathers and observed data are time-major,
 * sample (t, ir) at t*nr+ir; images are interior nx*nz, x-major.
 */
#ifndef QPSTD_H
#define QPSTD_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define QPSTD_OK 0
#define QPSTD_EINVAL (-1)    /* bad argument (sizes, indices, null pointers) */
#define QPSTD_ECUDA (-2)     /* CUDA runtime error (message in qpstd_last_error) */
#define QPSTD_ENOMEM (-3)    /* device allocation failed */
#define QPSTD_EREVOLVE (-4)  /* checkpoint schedule error (revolve info code) */
#define QPSTD_ENOTSUP (-5)   /* combination not built */

/* program kinds (the reference's four executables) */
#define QPSTD_APS 0   /* acoustic modeling            */
#define QPSTD_VAPS 1  /* constant-Q modeling          */
#define QPSTD_ARTM 2  /* acoustic RTM                 */
#define QPSTD_QRTM 3  /* Q-compensated RTM            */

/* step implementations */
#define QPSTD_FUSED 0  /* hand-written shared-memory line-FFT passes (default) */
#define QPSTD_PLAIN 1  /* cuFFT 2-D C2C + elementwise kernels, the reference's step order */

/* One shot on its padded (window + CPML) grid.  All pointers are host memory
 * owned by the caller and only read during the call. */
typedef struct qpstd_shot_desc {
    int kind;                 /* QPSTD_APS .. QPSTD_QRTM */
    int method;               /* QPSTD_FUSED or QPSTD_PLAIN */
    int nxx, nzz, pml;        /* padded grid (nx+2*pml, nz+2*pml) and CPML width */
    float dx, dz;             /* grid spacing (m) */
    float dt;                 /* time step (s); the reference reads ms and divides by 1000 */
    float fd;                 /* dominant frequency: CPML alpha_max = pi*fd (funca.c:230) */
    int nt;                   /* time samples (tmax) */
    const float *vp, *rho;    /* windowed, PML-expanded models, nxx*nzz */
    const float *bbx, *bbz;   /* staggered buoyancy, nxx*nzz (cal_bbx_bbz on the full model) */
    const float *gam, *lam, *vwd, *tao; /* constant-Q fields (transfermodel), VAPS/QRTM only */
    const float *rik;         /* source wavelet, nt */
    int xsg, zsg;             /* source grid index on the padded grid */
    int nr;                   /* receivers */
    const int *gxg, *gzg;     /* receiver grid indices on the padded grid */
    float etas, etar;         /* Q-RTM filter stabilisation (x 1e-6 inside, as the reference) */
    float taoc;               /* Q-RTM filter tau: max tau over the window (acsglw.cu:354-356) */
    int snaps;                /* RTM checkpoints (revolve snaps), 1..64 */
} qpstd_shot_desc;

/* Library / device status.  Thread-compatible: one caller per device. */
const char *qpstd_last_error(void);
int qpstd_version(void);

/* Modeling of one shot (aps / vaps).  gather: nt*nr floats, p after the
 * pressure update of each step at the receivers (acps4.cu:568,611-621).
 * state (optional, NULL to skip): the final p,vx,vz,fipx,fipz,fivxx,fivzz,aux,
 * 8*nxx*nzz floats.  Replaces the per-shot body of acforward (aps, vaps). */
int qpstd_model_shot(const qpstd_shot_desc *d, float *gather, float *state);

/* RTM of one shot (artm / qrtm).  obs: nt*nr observed data (direct arrival
 * already muted, removedirect).  img, ssg: nx*nz (interior) cross-correlation
 * image and first-sweep source illumination, before the Laplacian filter.
 * Replaces the per-shot body of acforward (artm, qrtm) up to filter_image. */
int qpstd_rtm_shot(const qpstd_shot_desc *d, const float *obs, float *img, float *ssg);

/* 5-point Laplacian image filter with the border zeroed, on the device
 * (filter_image, sgpstd-qrtm/acsglw.cu:1872; the reference's out-of-range
 * writes are not reproduced).  img, imgf: host nx*nz. */
int qpstd_filter_image(int nx, int nz, float dx, float dz, const float *img, float *imgf);

/* The CPML profiles the library applies for a grid (get_pml_parameters,
 * sgpstd-qmodeling/funca.c:223-340, evaluated in double and rounded): out holds
 * i_ax, i_bx, h_ax, h_bx (nxx each), then i_az, i_bz, h_az, h_bz (nzz each).
 * Host only.  The acforward shims compare the tables their caller computed with
 * these and warn when they differ (the library always applies its own). */
int qpstd_pml_profiles(int pml, float fd, int nxx, int nzz, float dx, float dz, float dt, float *out);

/* Source-normalised imaging condition out = img / (ssg + sigma2) on the
 * device (host nx*nz arrays): the reference leaves this step to the user after
 * summing img_sp / ssg_sp; sigma2 is the stabilisation (e.g. 1e-26). */
int qpstd_normalize_image(int nx, int nz, float sigma2, const float *img, const float *ssg, float *out);

/* ---- device-resident shot handle (inputs stay in HBM between calls) ---- */
typedef struct qpstd_shot qpstd_shot;

/* Uploads the models and builds all coefficient tables and FFT plans. */
int qpstd_shot_create(const qpstd_shot_desc *d, qpstd_shot **out);
int qpstd_shot_destroy(qpstd_shot *s);
/* 8*nxx*nzz host floats in the order of qpstd_model_shot's state. */
int qpstd_shot_set_state(qpstd_shot *s, const float *state);
int qpstd_shot_get_state(qpstd_shot *s, float *state);
/* Advance nsteps steps starting at step index t0 (source wavelet index).
 * gather (host, may be NULL): nsteps*nr floats. */
int qpstd_shot_advance(qpstd_shot *s, int t0, int nsteps, float *gather);
/* Same, leaving the gather in device memory (no host copy, no sync). */
int qpstd_shot_advance_device(qpstd_shot *s, int t0, int nsteps);
/* The same steps as a caller-driven pipeline (for streaming and timing):
 * begin() prepares the first step, each step(t, last) runs one time step at
 * source-wavelet index t (last=1 on the final one), end() completes the last
 * step.  Only after end() does the state equal the reference's. */
int qpstd_shot_pipeline_begin(qpstd_shot *s);
int qpstd_shot_pipeline_step(qpstd_shot *s, int t, int last);
int qpstd_shot_pipeline_end(qpstd_shot *s);
/* Number of kernels launched since the last advance / RTM / pipeline_begin. */
long long qpstd_shot_launch_count(const qpstd_shot *s);
/* Full RTM of the shot with the device-resident observed data uploaded by
 * qpstd_shot_set_obs; results stay on the device until qpstd_shot_get_image. */
int qpstd_shot_set_obs(qpstd_shot *s, const float *obs);
int qpstd_shot_rtm_device(qpstd_shot *s);
int qpstd_shot_get_image(qpstd_shot *s, float *img, float *ssg);
/* Forward steps the last RTM executed (revolve recompute included). */
long long qpstd_shot_forward_steps(const qpstd_shot *s);
/* Synchronise the shot's stream. */
int qpstd_shot_sync(qpstd_shot *s);
/* The shot's CUDA stream (cudaStream_t), for callers that order or time work on it. */
void *qpstd_shot_stream(qpstd_shot *s);

/* Per-launch timing: while on, every kernel launch of the shot is bracketed by
 * CUDA events on its stream; profile_read synchronises and returns, per kernel
 * kind, the summed milliseconds and the launch count, then clears the record. */
#define QPSTD_K_XPASS 0   /* x-line pass (real fields) */
#define QPSTD_K_ZPASS 1   /* z-line pass (real fields) */
#define QPSTD_K_XSPEC 2   /* x-line pass over z-spectra (2-D isotropic operators) */
#define QPSTD_K_OTHER 3   /* small helpers (checkpoint-0 source sample, filters) */
#define QPSTD_K_PLAIN 4   /* one whole plain-form step (cuFFT calls + elementwise kernels) */
#define QPSTD_K_XSPEC_EXACT 5 /* x-line pass over z-spectra on exact DFTs (Bluestein when nxx needs it) */
#define QPSTD_NKINDS 6
int qpstd_shot_set_profiling(qpstd_shot *s, int on);
int qpstd_shot_profile_read(qpstd_shot *s, int nkinds, double *ms, long long *count);

/* Facts about the transforms a created shot runs (for tests and tools); -1
 * for a null shot or an unknown key.  No counterpart in the reference, whose
 * cufftPlan2d chooses its own algorithm. */
#define QPSTD_INFO_X_CONV_M 0        /* length of the x convolution transform (separable operators) */
#define QPSTD_INFO_X_CONV_MAXRADIX 1 /* largest radix of that transform */
#define QPSTD_INFO_X_EXACT_M 2       /* inner length of the exact length-nxx DFT (Bluestein: >= 2nxx-1) */
#define QPSTD_INFO_X_EXACT_BLUE 3    /* 1 if the exact x DFT runs through Bluestein's identity */
#define QPSTD_INFO_X_SPEC_CONV 4     /* 1 if stationary 2-D symbols run as per-kz x convolutions */
#define QPSTD_INFO_Z_EXACT_M 5       /* inner length of the exact length-nzz DFT */
#define QPSTD_INFO_Z_EXACT_MAXRADIX 6
#define QPSTD_INFO_Z_CONV_M 7
long long qpstd_shot_info(const qpstd_shot *s, int key);

/* ---- batches: many resident shots advancing together ---------------------
 * The reference runs a rank's shots one after another (the shot loop of
 * acforward, sgpstd-qrtm/acsglw.cu:304).  A batch keeps all of them in HBM,
 * each with its own stream, and interleaves their revolve actions so their
 * kernels overlap.  Windows (nxx), nt and snaps may differ between shots. */
typedef struct qpstd_batch qpstd_batch;
int qpstd_batch_create(const qpstd_shot_desc *d, int nshots, qpstd_batch **out);
int qpstd_batch_destroy(qpstd_batch *b);
int qpstd_batch_size(const qpstd_batch *b);
/* The i-th shot (for qpstd_shot_set_obs / get_image / get_state ...). */
qpstd_shot *qpstd_batch_shot(qpstd_batch *b, int i);
int qpstd_batch_sync(qpstd_batch *b);
/* RTM of every shot; advances are enqueued `slice` steps at a time per shot.
 * First moves each shot to a new stream whose CUDA priority grows with the
 * shot's work (widest windows first), after the work already on its stream:
 * a stream taken from qpstd_shot_stream before this call is not the shot's
 * stream afterwards. */
int qpstd_batch_rtm_device(qpstd_batch *b, int slice);
int qpstd_batch_pipeline_begin(qpstd_batch *b);
int qpstd_batch_pipeline_step(qpstd_batch *b, int t, int last);
int qpstd_batch_pipeline_end(qpstd_batch *b);
/* One call with host buffers: obs[i] nt*nr, img[i] and ssg[i] nx*nz of shot i
 * (ssg may be NULL). */
int qpstd_rtm_batch(const qpstd_shot_desc *d, int nshots, const float *const *obs, float *const *img,
                    float *const *ssg);

/* Device bytes qpstd_shot_create would take for d (all buffers, RTM snapshot
 * pool included); -1 for an invalid descriptor. */
long long qpstd_shot_bytes(const qpstd_shot_desc *d);

/* ---- serving: continuous batching of shot requests ------------------------
 * No counterpart in the reference (its programs run a fixed shot list, one
 * shot at a time).  A server owns one device-memory arena (mem_budget bytes;
 * 0: 85 % of the free memory) and a worker thread that admits queued requests
 * in arrival order while a slot (max_active; 0: 64) and memory allow, runs each
 * admitted shot on its own stream in slices so later requests overlap with
 * running ones, and retires finished shots.  An RTM request is given the
 * largest revolve snapshot count, up to its d->snaps, that fits at admission;
 * the image is the one qpstd_rtm_shot gives with that count (qpstd_server_status
 * reports it).  A fused request whose window the fused passes cannot plan
 * (x lines beyond about 4600 points, z lines beyond about 2800) runs in the
 * plain form. */
typedef struct qpstd_server qpstd_server;
int qpstd_server_create(long long mem_budget, int max_active, qpstd_server **out);
/* Waits for every submitted request, then stops the worker. */
int qpstd_server_destroy(qpstd_server *sv);
/* Queues one shot; returns its request id (>= 0) or a negative status.
 * APS / VAPS: out0 = gather nt*nr (obs, out1 unused).  ARTM / QRTM: obs =
 * observed data nt*nr, out0 = image nx*nz, out1 = illumination nx*nz or NULL.
 * Every array d points at, and obs / out0 / out1, must stay valid until the
 * request is done. */
long long qpstd_server_submit(qpstd_server *sv, const qpstd_shot_desc *d, const float *obs, float *out0,
                              float *out1);
/* 0 queued, 1 running, 2 done, < 0 failed (status code).  latency_s: seconds
 * from submit to done (so far, while not done); snaps_used: the snapshot count
 * an RTM request ran with.  Either may be NULL. */
int qpstd_server_status(qpstd_server *sv, long long id, double *latency_s, int *snaps_used);
/* Blocks until request id is done (id < 0: every request submitted so far). */
int qpstd_server_wait(qpstd_server *sv, long long id);

/* ---- low-rank form of the constant-Q mixed-domain symbol -----------------
 * W(x,k) = sinc(vp dt k^(1+gam)/2) k^gam sqrt(1 + dt tau k^1.01/2), sinc(u) =
 * sin(u)/u, |k| on the half grid nxh x nzh (nxh = nxx/2+1, nzh = nzz/2+1,
 * k[0] = 1e-6, cal_k2dh, sgpstd-qmodeling/func.c:783).  Replaces acsglowrank2d
 * (sgpstd-qmodeling/sglowrank.c:148), whose call site is commented out in the
 * reference (sgpstd-qmodeling/acsglw.cu:367-389).  FP64 setup, seeded (the
 * reference seeds rand() from the clock).  Host only, no GPU needed.
 * vp, tao, gam: nxx*nzz.  Outputs (each may be NULL): U nxx*nzz x col,
 * V row x nxh*nzh, A col x row (double), jrr[col] chosen wavenumbers,
 * irr[row] chosen points. */
int qpstd_lowrank_decompose(int nxx, int nzz, float dx, float dz, float dt, const float *vp, const float *tao,
                            const float *gam, int row, int col, unsigned long long seed, float *U, float *V,
                            double *A, int *jrr, int *irr);
/* Exact row W(x_is, k) and its low-rank approximation, nxh*nzh floats each
 * (checka_error, sgpstd-qmodeling/sglowrank.c:61-101).  Host only. */
int qpstd_lowrank_check(int nxx, int nzz, float dx, float dz, float dt, int row, int col, const float *U,
                        const double *A, const float *V, const float *vp, const float *tao, const float *gam,
                        int is, float *We, float *Wa);
/* Runs a created fused constant-Q shot (VAPS / QRTM) in the low-rank form: the
 * pressure update becomes p += rho vp^2 dt W{div} -/+ dt tau aux (- modeling,
 * + Q-compensated RTM, as the power-expansion form), where W{div} = sum_a
 * U[x][a] sum_b A[a][b] Re F^-1[Vt_b F div] / N is the reference's dormant
 * low-rank operator (sgpstd-qmodeling/acsglw.cu:1375-1497) applied as its
 * dormant pressure update applies it (addsa_b_kernel, acsglw.cu:1542-1571; the
 * reference's call sites, acsglw.cu:367-389, are commented out, so this wiring
 * is this library's).  U, V, A as qpstd_lowrank_decompose returns them for the
 * shot's window (row, col <= 16).  The step then runs the low-rank x-spectral
 * pass and its z sum in place of the power expansion's three passes. */
int qpstd_shot_set_lowrank(qpstd_shot *s, int row, int col, const float *U, const float *V, const double *A);

/* Device operator out = sum_a U[x][a] sum_b A[a][b] Re F^-1[Vt_b F in](x) / N
 * (the reference's multv_kernel / sumlw_kernel / sumlw2_kernel,
 * sgpstd-qmodeling/acsglw.cu:1375-1497, with Vt_b = consist_Vt of V_b). */
typedef struct qpstd_lowrank qpstd_lowrank;
int qpstd_lowrank_create(int nxx, int nzz, int row, int col, const float *U, const float *V, const double *A,
                         qpstd_lowrank **out);
int qpstd_lowrank_destroy(qpstd_lowrank *h);
/* in, out: host nxx*nzz. */
int qpstd_lowrank_apply(qpstd_lowrank *h, const float *in, float *out);
/* d_in, d_out: device nxx*nzz; stream: cudaStream_t (NULL: the handle's own). No sync. */
int qpstd_lowrank_apply_device(qpstd_lowrank *h, const float *d_in, float *d_out, void *stream);

/* ---- acoustic steps without device allocation ---------------------------
 * No counterpart in the reference (its acforward allocates all device memory
 * itself).  For callers that cannot call cudaMalloc -- plug-ins that may only
 * use the buffers their host application hands them, hosts whose device memory
 * all belongs to a pool they do not own, latency-critical callers that may not
 * allocate (cudaFree synchronises the device).  Runs nsteps acoustic steps (aps / the source side of
 * artm) from step index t0, exactly as qpstd_shot_advance does, with every
 * scratch buffer and table in a static array of QPSTD_NOALLOC_FLOATS floats
 * (24 MiB) that each GPU loading the library keeps until exit; grids above
 * QPSTD_NOALLOC_MAX_POINTS points are rejected with QPSTD_EINVAL.
 * d: the shot (scalars, wavelet and receivers on the host; its model pointers
 *    are not read); vp, rho, bbx, bbz: device, nxx*nzz each; state: device,
 *    8*nxx*nzz (p, vx, vz, fipx, fipz, fivxx, fivzz, aux), advanced in place;
 *    gather: device nsteps*nr or NULL; stream: a cudaStream_t (NULL: legacy).
 * The first call on a device looks up the array's address (make it before any
 * stream capture).  Calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller. */
#define QPSTD_NOALLOC_FLOATS (6 * 1024 * 1024)
#define QPSTD_NOALLOC_MAX_POINTS (1024 * 1024)
int qpstd_ac_advance_noalloc(const qpstd_shot_desc *d, const float *vp, const float *rho, const float *bbx,
                             const float *bbz, float *state, int t0, int nsteps, float *gather, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* QPSTD_H */
