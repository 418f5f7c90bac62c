// acforward_common.h -- the shared per-shot body of the reference-signature
// acforward shims.
//
// The reference builds each program (aps, vaps, artm, qrtm) from a host main
// (parameters, MPI shot distribution, model files, coefficient tables) and one
// CUDA file whose extern "C" acforward time-steps the shots.  A shim object
// compiled from acforward_<program>.cpp has that acforward's exact signature;
// linked in place of the CUDA file (with libqpstd.so), the program's own main
// and host C helpers run unchanged.  Per shot the shim does what the
// reference's acforward does on the host -- window the models, place source and
// receivers, write the gather / read and mute the observed data, filter, mute
// and project the image -- and hands the time stepping to the C ABI.
//
// Differences: one GPU per process (GPU_N must be 1; the reference's MPI ranks
// each own a GPU); the coefficient tables the program passes (CPML profiles,
// shift and k-space symbols) are not read -- the library evaluates the same
// formulas in FP64 -- except that the CPML frequency, which acforward does not
// receive, is recovered from the interior CPML decay i_bx = exp(-dt pi fd).
#pragma once
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/qpstd.h"

// The program's struct MultiGPU (statement.h) begins with the shot table that
// its main fills before calling acforward; the shims read only this prefix.
struct MultiGPU {
    int *shotid;
    float *sxp;
    float *szp;
};

// Host helpers the program links (its funca.c / func.c), called as the
// reference's acforward calls them.
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

namespace qpshim {

// The grid, model and geometry arguments every acforward receives.
struct Common {
    int tmax;
    float dt;
    float *rik;
    int myid;
    float *gxp, *gzp;
    int nrmx, nx, nz, nxx, nzz, pml;
    float dx, dz, sroffmx, disx;
    int nxt, nzt;
    int *tracenum;
    float *i_bx;
    char *fname4, *fname5;
    float fd = 0.f;  // CPML frequency when known (the native programs); 0: recovered from i_bx
    int method = QPSTD_FUSED;
    // the caller's CPML profiles (i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz), when it passes them
    const float *cpml[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

inline void set_cpml(Common &c, const float *i_ax, const float *i_bx, const float *i_az, const float *i_bz,
                     const float *h_ax, const float *h_bx, const float *h_az, const float *h_bz) {
    const float *t[8] = {i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz};
    for (int k = 0; k < 8; k++) c.cpml[k] = t[k];
}

// The reference's acforward takes every coefficient table from its caller; the
// library computes them itself from the grid, dt and the CPML frequency.  Warns
// (stderr) when the caller's CPML profiles differ from the library's by more
// than 1e-4 of their largest value, i.e. when a modified main passes tables of
// another CPML, which the library would not apply.
inline void check_cpml(const Common &c, float fd) {
    if (!c.cpml[0]) return;
    std::vector<float> lib((size_t)4 * (c.nxx + c.nzz));
    if (qpstd_pml_profiles(c.pml, fd, c.nxx, c.nzz, c.dx, c.dz, c.dt, lib.data()) != QPSTD_OK) return;
    const char *names[8] = {"i_ax", "i_bx", "i_az", "i_bz", "h_ax", "h_bx", "h_az", "h_bz"};
    const int at[8] = {0, 1, 4, 5, 2, 3, 6, 7};  // positions in qpstd_pml_profiles' order
    for (int k = 0; k < 8; k++) {
        const bool x = (k == 0 || k == 1 || k == 4 || k == 5);
        const int n = x ? c.nxx : c.nzz;
        const size_t off = (at[k] < 4) ? (size_t)at[k] * c.nxx : (size_t)4 * c.nxx + (size_t)(at[k] - 4) * c.nzz;
        double dmax = 0.0, vmax = 0.0;
        for (int i = 0; i < n; i++) {
            dmax = std::max(dmax, std::fabs((double)c.cpml[k][i] - lib[off + i]));
            vmax = std::max(vmax, std::fabs((double)lib[off + i]));
        }
        if (dmax > 1e-4 * std::max(vmax, 1e-30))
            fprintf(stderr,
                    "warning: the %s table passed to acforward differs from the CPML profile libqpstd applies "
                    "(max difference %.3g of %.3g); the library uses get_pml_parameters with pml=%d, fd=%g\n",
                    names[k], dmax, vmax, c.pml, fd);
    }
}

// One shot on its window (sgpstd-qmodeling/acps4.cu:312-430).
struct Shot {
    int shotid = 0, nr = 0, xsg = 0, zsg = 0, lgest = 10000, rgest = -1;
    float xs = 0.f, zs = 0.f, mlx = 0.f;
    std::vector<float> f[8];  // vp, rho, bbx, bbz, gam, lam, vwd, tao
    std::vector<int> gxg, gzg;
};

// CPML frequency from the interior decay the program computed (i_bx = exp(-dt pi fd)).
inline float cpml_fd(const Common &c) {
    if (c.fd > 0.f || !c.i_bx) return c.fd;
    const float b = c.i_bx[c.nxx / 2];
    return (b > 0.f && b < 1.f) ? (float)(-std::log((double)b) / ((double)c.dt * 3.1415926)) : 0.f;
}

// Windows the given full models (null entries skipped) and places source and receivers.
inline bool window(const Common &c, MultiGPU *singpu, int ns, float *const *models, Shot &s) {
    s.shotid = singpu[0].shotid[ns];
    s.xs = singpu[0].sxp[ns];
    s.zs = singpu[0].szp[ns];
    printf("myid=%d shotid=%d nxx=%d nzz=%d xs=%f zs=%f\n", c.myid, s.shotid, c.nxx, c.nzz, s.xs, s.zs);
    s.mlx = s.xs - c.sroffmx - c.disx;
    const size_t N = (size_t)c.nxx * c.nzz;
    for (int k = 0; k < 8; k++) {
        s.f[k].clear();
        if (!models[k]) continue;
        s.f[k].assign(N, 0.f);
        select_part_model(c.pml, s.mlx, c.dx, c.nxt, c.nzt, c.nx, c.nz, c.nxx, c.nzz, models[k], s.f[k].data());
        expand_pml_areas(c.nx, c.nz, c.nxx, c.nzz, c.pml, s.f[k].data());
    }
    s.zsg = (int)(s.zs / c.dz + 0.5) + c.pml;
    s.xsg = (int)((c.sroffmx + c.disx) / c.dx + 0.5) + c.pml;
    if (s.xsg < 0 || s.xsg >= c.nxx || s.zsg < 0 || s.zsg >= c.nzz) {
        printf("%d shot grid index exceeds model!\n", s.shotid);
        return false;
    }
    s.nr = c.tracenum[s.shotid];
    input_geophone_pos(s.shotid, s.nr, c.gxp, c.fname4);
    input_geophone_pos(s.shotid, s.nr, c.gzp, c.fname5);
    s.gxg.assign(s.nr, 0);
    s.gzg.assign(s.nr, 0);
    s.lgest = 10000;
    s.rgest = -1;
    for (int i = 0; i < s.nr; i++) {
        s.gzg[i] = (int)(c.gzp[i] / c.dz + 0.5) + c.pml;
        if (c.gxp[i] >= s.xs) s.gxg[i] = s.xsg + (int)((c.gxp[i] - s.xs) / c.dx + 0.5);
        else s.gxg[i] = s.xsg - (int)((s.xs - c.gxp[i]) / c.dx + 0.5);
        if (s.gxg[i] < c.pml) {
            printf("warning: receiver x grid index in left pml area!\n");
            s.gxg[i] = c.pml;
        }
        if (s.gxg[i] >= c.nxx - c.pml) {
            printf("warning: receiver x grid index in right pml area!\n");
            s.gxg[i] = c.nxx - c.pml - 1;
        }
        s.rgest = std::max(s.rgest, s.gxg[i]);
        s.lgest = std::min(s.lgest, s.gxg[i]);
    }
    return true;
}

inline qpstd_shot_desc describe(const Common &c, Shot &s, int kind, float fd) {
    qpstd_shot_desc d;
    memset(&d, 0, sizeof(d));
    d.kind = kind;
    d.method = c.method;
    d.nxx = c.nxx;
    d.nzz = c.nzz;
    d.pml = c.pml;
    d.dx = c.dx;
    d.dz = c.dz;
    d.dt = c.dt;
    d.fd = fd;
    d.nt = c.tmax;
    float **p[8] = {(float **)&d.vp, (float **)&d.rho, (float **)&d.bbx, (float **)&d.bbz,
                    (float **)&d.gam, (float **)&d.lam, (float **)&d.vwd, (float **)&d.tao};
    for (int k = 0; k < 8; k++) *p[k] = s.f[k].empty() ? nullptr : s.f[k].data();
    d.rik = c.rik;
    d.xsg = s.xsg;
    d.zsg = s.zsg;
    d.nr = s.nr;
    d.gxg = s.gxg.data();
    d.gzg = s.gzg.data();
    return d;
}

inline void report(int rc, int shotid) {
    if (rc) printf("shot %d: libqpstd error %d: %s\n", shotid, rc, qpstd_last_error());
}

// Appends float records to files on a background thread, so that snapshot
// writes overlap the next steps on the GPU.  The destructor drains the queue.
class AsyncWriter {
public:
    AsyncWriter() : th_([this] { run(); }) {}
    ~AsyncWriter() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    void append(const std::string &path, std::vector<float> rec) {
        {
            std::lock_guard<std::mutex> g(m_);
            q_.push_back({path, std::move(rec)});
        }
        cv_.notify_all();
    }

private:
    void run() {
        for (;;) {
            std::pair<std::string, std::vector<float>> job;
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [this] { return stop_ || !q_.empty(); });
                if (q_.empty()) return;
                job = std::move(q_.front());
                q_.pop_front();
            }
            FILE *f = fopen(job.first.c_str(), "ab");
            if (f) {
                fwrite(job.second.data(), sizeof(float), job.second.size(), f);
                fclose(f);
            }
        }
    }
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<std::pair<std::string, std::vector<float>>> q_;
    bool stop_ = false;
    std::thread th_;
};

// Gather of a modeled shot to "../obsdata/<prefix><shotid>_<nr>.bin" (time-major nt x nr).
inline void write_gather(const Common &c, const Shot &s, const float *gather, const char *recpre) {
    char name[256];
    snprintf(name, sizeof name, "../obsdata/%s%d_%d.bin", recpre, s.shotid, s.nr);
    FILE *fr = fopen(name, "wb");
    if (!fr) {
        printf("shot %d: cannot write %s\n", s.shotid, name);
        return;
    }
    fwrite(gather, sizeof(float), (size_t)c.tmax * s.nr, fr);
    fclose(fr);
}

// One modeled shot with the interior p of every tenth step appended to
// "../obsdata/<snap><shotid>_<nz>_<nx>.bin" (sgpstd-qmodeling/acps4.cu:624-640).
inline int model_with_snapshots(const Common &c, const Shot &s, const qpstd_shot_desc &d, float *gather,
                                const char *snappre, AsyncWriter &wr) {
    char snap[256];
    snprintf(snap, sizeof snap, "../obsdata/%s%d_%d_%d.bin", snappre, s.shotid, c.nz, c.nx);
    FILE *fs = fopen(snap, "wb");
    if (fs) fclose(fs);
    qpstd_shot *h = nullptr;
    int rc = qpstd_shot_create(&d, &h);
    std::vector<float> st((size_t)8 * c.nxx * c.nzz);
    // steps [0], [1..10], [11..20], ...: the state after every t % 10 == 0
    for (int t0 = 0; !rc && t0 < c.tmax;) {
        const int n = (t0 == 0) ? 1 : std::min(10, c.tmax - t0);
        rc = qpstd_shot_advance(h, t0, n, gather + (size_t)t0 * s.nr);
        const int tl = t0 + n - 1;
        if (!rc && tl % 10 == 0 && !(rc = qpstd_shot_get_state(h, st.data()))) {
            std::vector<float> rec((size_t)c.nx * c.nz);
            for (int ix = 0; ix < c.nx; ix++)
                std::copy(&st[(size_t)(ix + c.pml) * c.nzz + c.pml], &st[(size_t)(ix + c.pml) * c.nzz + c.pml + c.nz],
                          &rec[(size_t)ix * c.nz]);
            wr.append(snap, std::move(rec));
        }
        t0 += n;
    }
    qpstd_shot_destroy(h);
    return rc;
}

// Modeling: gather to "../obsdata/<prefix><shotid>_<nr>.bin"; with flagout the
// interior p of every tenth step appended to "../obsdata/<snap><shotid>_<nz>_<nx>.bin"
// (sgpstd-qmodeling/acps4.cu:568-640).
inline void model(const Common &c, MultiGPU *singpu, int nshot, float *const *models, int kind, int flagout,
                  const char *recpre, const char *snappre) {
    const float fd = cpml_fd(c);
    check_cpml(c, fd);
    AsyncWriter wr;
    for (int ns = 0; ns < nshot; ns++) {
        Shot s;
        if (!window(c, singpu, ns, models, s)) continue;
        qpstd_shot_desc d = describe(c, s, kind, fd);
        std::vector<float> gather((size_t)c.tmax * std::max(s.nr, 1), 0.f);
        const int rc = flagout ? model_with_snapshots(c, s, d, gather.data(), snappre, wr)
                               : qpstd_model_shot(&d, gather.data(), nullptr);
        report(rc, s.shotid);
        write_gather(c, s, gather.data(), recpre);
    }
}

// RTM: observed data from "<recname><shotid>_<nr>.bin" with the direct wave
// removed, the image filtered, muted outside the receiver aperture, projected
// onto the model and summed into img_sp / ssg_sp (sgpstd-qrtm/acsglw.cu:409-420,
// 1041-1079).
// RTM parameters beyond the common ones.
struct RtmArgs {
    int kind, snapnum;
    float fobs, v0, etas, etar;
    const char *recname;
};

// One RTM shot made ready: window, observed data with the direct wave removed
// (obs, nt x nr) and the shot descriptor (pointing into s).
inline bool rtm_prepare(const Common &c, MultiGPU *singpu, int ns, float *const *models, const RtmArgs &a, Shot &s,
                        std::vector<float> &obs, qpstd_shot_desc &d) {
    if (!window(c, singpu, ns, models, s)) return false;
    obs.assign((size_t)c.tmax * std::max(s.nr, 1), 0.f);
    char name[256];
    snprintf(name, sizeof name, "%s%d_%d.bin", a.recname, s.shotid, s.nr);
    FILE *fr = fopen(name, "rb");
    if (!fr || fread(obs.data(), sizeof(float), (size_t)c.tmax * s.nr, fr) != (size_t)c.tmax * s.nr)
        printf("shot %d: cannot read %s\n", s.shotid, name);
    if (fr) fclose(fr);
    removedirect(c.nrmx, c.tmax, s.nr, c.dt, a.fobs, s.xs, s.zs, c.gxp, c.gzp, a.v0, obs.data());
    d = describe(c, s, a.kind, cpml_fd(c));
    d.snaps = a.snapnum;
    d.etas = a.etas;
    d.etar = a.etar;
    if (a.kind == QPSTD_QRTM) d.taoc = get_max_tao(c.nxx, c.nzz, s.f[7].data());  // acsglw.cu:354-356
    return true;
}

// One shot's image (nx x nz) filtered, muted outside the receiver aperture and
// projected onto the model, summed with its illumination into img_sp / ssg_sp.
inline int rtm_accumulate(const Common &c, const Shot &s, const float *img, const float *ssg, float *img_sp,
                          float *ssg_sp) {
    const size_t NI = (size_t)c.nx * c.nz, NT = (size_t)c.nxt * c.nzt;
    std::vector<float> imgf(NI), ssgw(ssg, ssg + NI), img_pj(NT, 0.f), ssg_pj(NT, 0.f);
    const int rc = qpstd_filter_image(c.nx, c.nz, c.dx, c.dz, img, imgf.data());
    if (rc) return rc;
    const int lg = s.lgest - c.pml, rg = s.rgest - c.pml;
    for (int j = 0; j < c.nz; j++) {
        for (int i = 0; i < lg; i++) imgf[(size_t)i * c.nz + j] = 0.f;
        for (int i = std::max(rg, 0); i < c.nx; i++) imgf[(size_t)i * c.nz + j] = 0.f;
    }
    projectomodel(c.pml, s.mlx, c.dx, c.nxt, c.nzt, c.nx, c.nz, c.nxx, c.nzz, img_pj.data(), imgf.data());
    projectomodel(c.pml, s.mlx, c.dx, c.nxt, c.nzt, c.nx, c.nz, c.nxx, c.nzz, ssg_pj.data(), ssgw.data());
    for (size_t i = 0; i < NT; i++) {
        img_sp[i] += img_pj[i];
        ssg_sp[i] += ssg_pj[i];
    }
    return QPSTD_OK;
}

inline void rtm(const Common &c, MultiGPU *singpu, int nshot, float *const *models, int kind, int snapnum,
                float *img_sp, float *ssg_sp, float fobs, float v0, float etas, float etar, const char *recname) {
    const RtmArgs a{kind, snapnum, fobs, v0, etas, etar, recname};
    check_cpml(c, cpml_fd(c));
    const size_t NI = (size_t)c.nx * c.nz;
    std::vector<float> img(NI), ssg(NI), obs;
    for (int ns = 0; ns < nshot; ns++) {
        Shot s;
        qpstd_shot_desc d;
        if (!rtm_prepare(c, singpu, ns, models, a, s, obs, d)) continue;
        int rc = qpstd_rtm_shot(&d, obs.data(), img.data(), ssg.data());
        if (!rc) rc = rtm_accumulate(c, s, img.data(), ssg.data(), img_sp, ssg_sp);
        report(rc, s.shotid);
    }
}

inline bool one_gpu(int GPU_N) {
    if (GPU_N == 1) return true;
    printf("acforward (libqpstd): one GPU per process; GPU_N = %d is not supported\n", GPU_N);
    return false;
}

}  // namespace qpshim
