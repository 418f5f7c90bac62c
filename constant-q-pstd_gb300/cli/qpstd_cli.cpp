// qpstd_cli.cpp -- the native programs over libqpstd.
//
//   qpstd aps|vaps|artm|qrtm [options]   the reference's four programs
//   qpstd geometry [options]              geometry/geometry2d.c
//   qpstd sum OUT IN...                   element-wise sum of float32 files
//
// A copy or link of the executable named aps, vaps, artm, qrtm or geometry runs
// that program.  Each program reads the parameter file its reference
// counterpart reads (../input/<name>.txt relative to the working directory),
// the files it names, and writes the same outputs: ../obsdata/reca<id>_<nr>.bin
// / recva<id>_<nr>.bin gathers (and snapa / snapva snapshots) for modeling,
// RTM.BIN / QRTM.BIN (image then illumination, nxt x nzt each) for migration.
//
// The reference distributes shots over MPI ranks with one or more GPUs each
// (acousticsgps4.c:254-293).  Here a process drives one GPU; processes find
// their rank from the launcher's environment (RANK / WORLD_SIZE, Open MPI,
// PMI or Slurm variables) or --rank / --nranks, run their contiguous share of
// the shots, and with more than one process write <image>.rank<r>; `qpstd sum`
// adds those files (the reference's MPI_Reduce, sgpstd-qrtm/acrtmain.c:472).
//
// Within a process the shots run concurrently through the shot server (one
// stream per admitted shot), or one after another with --serial.  Snapshot
// output (flagout = 1) runs shot by shot.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "../../include/qpstd.h"
#include "../shims/acforward_common.h"
#include "programs.h"

namespace {

using qpcli::Program;

struct Options {
    std::string params;  // parameter file (default: the program's)
    std::string dir;     // geometry output directory
    std::string out;     // image file of RTM (default RTM.BIN / QRTM.BIN)
    int pml = 10;        // CPML width in cells (the reference's mains: #define pml 10)
    int rank = -1, nranks = -1;
    bool serial = false;
    bool dry_run = false;  // set up and report the windows, run nothing on the GPU
    int max_active = 0;
    double mem_gb = 0.0;
    int method = QPSTD_FUSED;
};

int env_int(std::initializer_list<const char *> names, int dflt) {
    for (const char *n : names) {
        const char *v = std::getenv(n);
        if (v && *v) return std::atoi(v);
    }
    return dflt;
}

template <class T>
bool read_array(const std::string &path, size_t n, std::vector<T> &out, const char *what) {
    out.assign(n, T());
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::printf("Cannot open the %s file %s !\n", what, path.c_str());
        return false;
    }
    const size_t got = std::fread(out.data(), sizeof(T), n, f);
    std::fclose(f);
    if (got != n) {
        std::printf("%s: %zu of %zu values\n", path.c_str(), got, n);
        return false;
    }
    return true;
}

bool write_file(const std::string &path, const std::vector<const std::vector<float> *> &parts) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    bool ok = true;
    for (const auto *p : parts) ok = ok && std::fwrite(p->data(), sizeof(float), p->size(), f) == p->size();
    std::fclose(f);
    return ok;
}

std::vector<char> cstr(const std::string &s) {
    std::vector<char> v(s.begin(), s.end());
    v.push_back('\0');
    return v;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// One shot in flight on the server; it stays at a fixed address (deque) while
// the server holds pointers into it.
struct Job {
    std::unique_ptr<qpshim::Shot> s{new qpshim::Shot()};
    qpstd_shot_desc d{};
    std::vector<float> obs, out0, out1;
    long long id = -1;
};

int run_program(Program p, const Options &o) {
    using namespace qpcli;
    const bool visco = (p == qpcli::VAPS || p == qpcli::QRTM), rtm = (p == qpcli::ARTM || p == qpcli::QRTM);
    const int kinds[4] = {QPSTD_APS, QPSTD_VAPS, QPSTD_ARTM, QPSTD_QRTM};
    const int kind = kinds[p];
    Params par;
    std::string err;
    const std::string pfile = o.params.empty() ? default_params(p) : o.params;
    if (!read_params(p, pfile, par, err)) {
        std::printf("%s\n", err.c_str());
        return 1;
    }
    const int nranks = o.nranks > 0 ? o.nranks : env_int({"WORLD_SIZE", "OMPI_COMM_WORLD_SIZE", "PMI_SIZE", "SLURM_NTASKS"}, 1);
    const int rank = o.rank >= 0 ? o.rank : env_int({"RANK", "OMPI_COMM_WORLD_RANK", "PMI_RANK", "SLURM_PROCID"}, 0);
    if (nranks < 1 || rank < 0 || rank >= nranks) {
        std::printf("bad rank %d of %d\n", rank, nranks);
        return 1;
    }
    const int shotnum = par.shotnum, tmax = par.tmax, nxt = par.nxt, nzt = par.nzt;
    if (shotnum < 1 || tmax < 1 || nxt < 1 || nzt < 1) {
        std::printf("bad sizes in %s\n", pfile.c_str());
        return 1;
    }
    const float dt = (float)(par.dt / 1000.0);
    const size_t NT = (size_t)nxt * nzt;
    std::vector<int> tracenum;
    std::vector<float> shotxp, shotzp, vpt, rhot, qpt;
    if (!read_array(par.trace, shotnum, tracenum, "tracenumber") || !read_array(par.shotx, shotnum, shotxp, "shot x position") ||
        !read_array(par.shotz, shotnum, shotzp, "shot z position") || !read_array(par.vp, NT, vpt, "velocity") ||
        !read_array(par.rho, NT, rhot, "density") || (visco && !read_array(par.qp, NT, qpt, "Qp")))
        return 1;
    float vmax, vmin;
    get_max_min((int)NT, vpt.data(), &vmax, &vmin);
    std::printf(" CFL number= %f %f %f\n", cfl_number(vmax, dt, par.dx, par.dz), vmax, vmin);

    std::vector<float> bbxt(NT), bbzt(NT), gamt, lamt, vwdt, taot;
    cal_bbx_bbz(nxt, nzt, rhot.data(), bbxt.data(), bbzt.data());
    if (visco) {
        gamt.resize(NT), lamt.resize(NT), vwdt.resize(NT), taot.resize(NT);
        transfermodel((int)NT, par.fd, par.fo, vpt.data(), qpt.data(), gamt.data(), lamt.data(), vwdt.data(),
                      taot.data());
    }
    std::vector<float> rik(tmax);
    rik_cal(tmax, dt, par.fd, par.flagsource, rik.data());

    int first = 0, nshot = 0;
    distribute(shotnum, nranks, rank, &first, &nshot);
    if (rank == nranks - 1) std::printf("Run total shot number is %d\n", first + nshot);
    const float xmax = (float)(nxt - 1) * par.dx, zmax = (float)(nzt - 1) * par.dz;
    std::vector<int> shotid(nshot);
    std::vector<float> sxp(nshot), szp(nshot);
    for (int j = 0; j < nshot; j++) {
        const int is = first + j;
        shotid[j] = is;
        sxp[j] = shotxp[is];
        szp[j] = shotzp[is];
        if (shotxp[is] < 0.f || shotxp[is] > xmax) return std::printf("%d shot x exceeds model!\n", is), 1;
        if (shotzp[is] < 0.f || shotzp[is] > zmax) return std::printf("%d shot z exceeds model!\n", is), 1;
    }
    int nrmx = -1;
    for (int v : tracenum) nrmx = std::max(nrmx, v);
    std::vector<float> gxp(std::max(nrmx, 1)), gzp(std::max(nrmx, 1));
    std::vector<char> fname4 = cstr(par.gxp), fname5 = cstr(par.gzp), recname = cstr(par.rec);
    float sroffmx = -1.0f;
    for (int i = first; i < first + nshot; i++) {
        const int nr = tracenum[i];
        input_geophone_pos(i, nr, gxp.data(), fname4.data());
        input_geophone_pos(i, nr, gzp.data(), fname5.data());
        float xrp, xlp, zrp, zlp;
        get_max_min(nr, gxp.data(), &xrp, &xlp);
        get_max_min(nr, gzp.data(), &zrp, &zlp);
        if (xlp < 0.f || xrp > xmax) return std::printf("%d shot receiver x exceeds model!\n", i), 1;
        if (zlp < 0.f || zrp > zmax) return std::printf("%d shot receiver z exceeds model!\n", i), 1;
        const float off = std::max(std::fabs(xrp - shotxp[i]), std::fabs(shotxp[i] - xlp));
        sroffmx = std::max(sroffmx, off);
    }
    const int nx = window_width(sroffmx, par.disx, par.dx), nz = nzt;
    const int nxx = nx + 2 * o.pml, nzz = nz + 2 * o.pml;
    std::printf("rank %d of %d: shots %d..%d, window nx=%d nz=%d, padded %d x %d, nt=%d\n", rank, nranks, first,
                first + nshot - 1, nx, nz, nxx, nzz, tmax);
    if (o.dry_run) return 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        std::printf("no CUDA device\n");
        return 1;
    }
    const int local = env_int({"LOCAL_RANK", "OMPI_COMM_WORLD_LOCAL_RANK", "MPI_LOCALRANKID", "SLURM_LOCALID"}, rank);
    cudaSetDevice(local % ndev);
    std::printf(" Process %d of %d on GPU %d of %d running...\n\n", rank, nranks, local % ndev, ndev);

    qpshim::Common c{tmax, dt, rik.data(), rank, gxp.data(), gzp.data(), nrmx, nx, nz, nxx, nzz, o.pml, par.dx,
                     par.dz, sroffmx, par.disx, nxt, nzt, tracenum.data(), nullptr, fname4.data(), fname5.data(),
                     par.fd, o.method};
    MultiGPU singpu{shotid.data(), sxp.data(), szp.data()};
    float *models[8] = {vpt.data(), rhot.data(), bbxt.data(), bbzt.data(), nullptr, nullptr, nullptr, nullptr};
    if (visco) models[4] = gamt.data(), models[5] = lamt.data(), models[6] = vwdt.data(), models[7] = taot.data();
    const char *recpre = visco ? "recva" : "reca", *snappre = visco ? "snapva" : "snapa";
    const qpshim::RtmArgs ra{kind, par.snapnum, par.fd, par.v0, par.etas, par.etar, recname.data()};
    std::vector<float> img_sp(rtm ? NT : 0, 0.f), ssg_sp(rtm ? NT : 0, 0.f);

    const double t0 = now_s();
    int failed = 0;
    if (nshot > 0 && (o.serial || (!rtm && par.flagout))) {
        if (rtm) qpshim::rtm(c, &singpu, nshot, models, kind, par.snapnum, img_sp.data(), ssg_sp.data(), par.fd,
                             par.v0, par.etas, par.etar, recname.data());
        else qpshim::model(c, &singpu, nshot, models, kind, par.flagout, recpre, snappre);
    } else if (nshot > 0) {
        qpstd_server *sv = nullptr;
        int rc = qpstd_server_create((long long)(o.mem_gb * 1e9), o.max_active, &sv);
        if (rc) {
            std::printf("shot server: %s\n", qpstd_last_error());
            return 1;
        }
        const size_t window = (size_t)std::max(4, 2 * (o.max_active > 0 ? o.max_active : 16));
        std::deque<Job> jobs;
        // results are taken in shot order, so the image sum is the serial one
        auto finish = [&](Job &j) {
            int st = qpstd_server_wait(sv, j.id), snaps = 0;
            qpstd_server_status(sv, j.id, nullptr, &snaps);
            if (!st && rtm) st = qpshim::rtm_accumulate(c, *j.s, j.out0.data(), j.out1.data(), img_sp.data(),
                                                        ssg_sp.data());
            if (!st && !rtm) qpshim::write_gather(c, *j.s, j.out0.data(), recpre);
            if (!st && rtm && snaps != j.d.snaps)
                std::printf("shot %d: ran with %d checkpoints of %d (device memory)\n", j.s->shotid, snaps, j.d.snaps);
            if (st) failed++;
            qpshim::report(st, j.s->shotid);
        };
        for (int ns = 0; ns < nshot; ns++) {
            jobs.emplace_back();
            Job &j = jobs.back();
            bool ok;
            if (rtm) {
                ok = qpshim::rtm_prepare(c, &singpu, ns, models, ra, *j.s, j.obs, j.d);
                j.out0.assign((size_t)nx * nz, 0.f);
                j.out1.assign((size_t)nx * nz, 0.f);
            } else {
                ok = qpshim::window(c, &singpu, ns, models, *j.s);
                if (ok) j.d = qpshim::describe(c, *j.s, kind, par.fd);
                j.out0.assign((size_t)tmax * std::max(j.s->nr, 1), 0.f);
            }
            if (ok) {
                j.id = qpstd_server_submit(sv, &j.d, rtm ? j.obs.data() : nullptr, j.out0.data(),
                                           rtm ? j.out1.data() : nullptr);
                if (j.id < 0) qpshim::report((int)j.id, j.s->shotid);
            }
            if (!ok || j.id < 0) {
                failed++;
                jobs.pop_back();
                continue;
            }
            while (jobs.size() >= window) {
                finish(jobs.front());
                jobs.pop_front();
            }
        }
        for (; !jobs.empty(); jobs.pop_front()) finish(jobs.front());
        qpstd_server_destroy(sv);
    }
    std::printf("The cost of the run time is %f seconds\n", now_s() - t0);

    if (rtm) {
        std::string out = o.out.empty() ? (p == qpcli::QRTM ? "QRTM.BIN" : "RTM.BIN") : o.out;
        if (nranks > 1) out += ".rank" + std::to_string(rank);
        if (!write_file(out, {&img_sp, &ssg_sp})) {
            std::printf("cannot write %s\n", out.c_str());
            return 1;
        }
    }
    return failed ? 2 : 0;
}

int run_geometry(const Options &o) {
    qpcli::GeometryParams g;
    std::string err;
    if (!qpcli::read_geometry_params(o.params.empty() ? "parameters.txt" : o.params, g, err) ||
        !qpcli::write_geometry(g, o.dir, err, true)) {
        std::printf("%s\n", err.c_str());
        return 1;
    }
    return 0;
}

int run_sum(int argc, char **argv) {
    if (argc < 2) {
        std::printf("usage: qpstd sum OUT IN...\n");
        return 1;
    }
    std::vector<float> acc, part;
    for (int i = 1; i < argc; i++) {
        FILE *f = std::fopen(argv[i], "rb");
        if (!f) return std::printf("cannot open %s\n", argv[i]), 1;
        std::fseek(f, 0, SEEK_END);
        const long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        part.assign((size_t)std::max(bytes, 0L) / sizeof(float), 0.f);
        const size_t got = std::fread(part.data(), sizeof(float), part.size(), f);
        std::fclose(f);
        if (got != part.size() || (i > 1 && part.size() != acc.size()))
            return std::printf("%s: size differs from %s\n", argv[i], argv[1]), 1;
        if (i == 1) acc.assign(part.size(), 0.f);
        for (size_t k = 0; k < acc.size(); k++) acc[k] += part[k];
    }
    return write_file(argv[0], {&acc}) ? 0 : (std::printf("cannot write %s\n", argv[0]), 1);
}

void usage() {
    std::printf(
        "usage: qpstd aps|vaps|artm|qrtm [--params FILE] [--pml N] [--rank R --nranks N] [--serial]\n"
        "                               [--max-active K] [--mem-gb G] [--plain] [--out FILE] [--dry-run]\n"
        "       qpstd geometry [--params FILE] [--dir DIR]\n"
        "       qpstd sum OUT IN...\n");
}

}  // namespace

int main(int argc, char **argv) {
    // shots run on one stream each: 32 hardware work queues (the default is 8);
    // read when the CUDA context is created, so before any CUDA call
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    std::string self = argv[0];
    const size_t slash = self.find_last_of('/');
    if (slash != std::string::npos) self = self.substr(slash + 1);
    std::string cmd = self;
    int a = 1;
    const char *progs[] = {"aps", "vaps", "artm", "qrtm", "geometry"};
    bool named = false;
    for (const char *pn : progs) named = named || self == pn;
    if (!named) {
        if (argc < 2) return usage(), 1;
        cmd = argv[1];
        a = 2;
    }
    if (cmd == "sum") return run_sum(argc - a, argv + a);
    Options o;
    for (; a < argc; a++) {
        const std::string k = argv[a];
        const bool has = a + 1 < argc;
        if (k == "--params" && has) o.params = argv[++a];
        else if (k == "--dir" && has) o.dir = argv[++a];
        else if (k == "--out" && has) o.out = argv[++a];
        else if (k == "--pml" && has) o.pml = std::atoi(argv[++a]);
        else if (k == "--rank" && has) o.rank = std::atoi(argv[++a]);
        else if (k == "--nranks" && has) o.nranks = std::atoi(argv[++a]);
        else if (k == "--max-active" && has) o.max_active = std::atoi(argv[++a]);
        else if (k == "--mem-gb" && has) o.mem_gb = std::atof(argv[++a]);
        else if (k == "--serial") o.serial = true;
        else if (k == "--dry-run") o.dry_run = true;
        else if (k == "--plain") o.method = QPSTD_PLAIN;
        else return usage(), 1;
    }
    if (o.pml < 1) return std::printf("--pml must be positive\n"), 1;
    if (cmd == "geometry") return run_geometry(o);
    for (int p = 0; p < 4; p++)
        if (cmd == progs[p]) return run_program((Program)p, o);
    usage();
    return 1;
}
