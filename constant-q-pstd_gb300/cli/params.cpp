// params.cpp -- parameter files of the four programs and of the geometry
// generator, and the geometry files themselves.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "programs.h"

namespace qpcli {

const char *default_params(Program p) {
    static const char *names[4] = {"../input/ac2drealmodeling.txt", "../input/visac2drealmodeling.txt",
                                   "../input/ac2drtm.txt", "../input/visac2drtm.txt"};
    return names[p];
}

const char *program_name(Program p) {
    static const char *names[4] = {"aps", "vaps", "artm", "qrtm"};
    return names[p];
}

namespace {

// The reference's readers alternate fgets (one label line) with fscanf of one
// value, skipping white space (blank lines included) on both sides of it.
class LabelledValues {
public:
    explicit LabelledValues(std::string text) : t_(std::move(text)) {}

    // next value as a token; false at the end of the text
    bool next(std::string &tok) {
        skip_ws();
        if (i_ >= t_.size()) return false;
        while (i_ < t_.size() && t_[i_] != '\n') i_++;  // the label line
        if (i_ < t_.size()) i_++;
        skip_ws();
        const size_t b = i_;
        while (i_ < t_.size() && !is_ws(t_[i_])) i_++;
        tok = t_.substr(b, i_ - b);
        return !tok.empty();
    }

private:
    static bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
    void skip_ws() {
        while (i_ < t_.size() && is_ws(t_[i_])) i_++;
    }
    std::string t_;
    size_t i_ = 0;
};

constexpr FieldKind I = FIELD_INT, F = FIELD_FLOAT, S = FIELD_STRING;

bool read_text(const std::string &path, std::string &text, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::ostringstream ss;
    ss << f.rdbuf();
    text = ss.str();
    return true;
}

bool parse(const std::string &path, const std::vector<Field> &fields, std::string &err) {
    std::string text;
    if (!read_text(path, text, err)) return false;
    LabelledValues lv(text);
    for (const Field &f : fields) {
        std::string tok;
        if (!lv.next(tok)) {
            err = path + ": missing value for " + f.what;
            return false;
        }
        char *end = nullptr;
        if (f.k == I) {
            const long v = std::strtol(tok.c_str(), &end, 10);
            if (end == tok.c_str()) {
                err = path + ": bad integer '" + tok + "' for " + f.what;
                return false;
            }
            *static_cast<int *>(f.p) = (int)v;
        } else if (f.k == F) {
            const float v = std::strtof(tok.c_str(), &end);
            if (end == tok.c_str()) {
                err = path + ": bad number '" + tok + "' for " + f.what;
                return false;
            }
            *static_cast<float *>(f.p) = v;
        } else {
            *static_cast<std::string *>(f.p) = tok;
        }
    }
    return true;
}

}  // namespace

std::vector<Field> param_layout(Program p, Params &o) {
    const bool visco = (p == VAPS || p == QRTM), rtm = (p == ARTM || p == QRTM);
    std::vector<Field> f = {{I, &o.shotnum, "shot number"}, {I, &o.tmax, "time samples"},
                            {F, &o.dt, "time step"},        {F, &o.fd, "dominant frequency"}};
    if (visco) f.push_back({F, &o.fo, "reference frequency"});
    f.insert(f.end(), {{I, &o.nxt, "nx"}, {I, &o.nzt, "nz"}, {F, &o.dx, "dx"}, {F, &o.dz, "dz"},
                       {F, &o.disx, "extended distance"}});
    if (rtm) f.push_back({F, &o.v0, "direct-wave velocity"});
    if (p == QRTM) f.insert(f.end(), {{F, &o.etas, "source stabilisation"}, {F, &o.etar, "receiver stabilisation"}});
    f.insert(f.end(), {{S, &o.trace, "trace number file"}, {S, &o.shotx, "shot x file"}, {S, &o.shotz, "shot z file"},
                       {S, &o.gxp, "receiver x prefix"}, {S, &o.gzp, "receiver z prefix"}, {S, &o.vp, "vp file"},
                       {S, &o.rho, "density file"}});
    if (visco) f.push_back({S, &o.qp, "Qp file"});
    if (rtm) f.push_back({S, &o.rec, "observed data prefix"});
    if (!rtm) f.push_back({I, &o.flagout, "snapshot flag"});
    f.push_back({I, &o.flagsource, "source flag"});
    if (rtm) f.push_back({I, &o.snapnum, "checkpoint number"});
    return f;
}

bool read_params(Program p, const std::string &path, Params &o, std::string &err) {
    return parse(path, param_layout(p, o), err);
}

bool read_geometry_params(const std::string &path, GeometryParams &g, std::string &err) {
    return parse(path,
                 {{I, &g.shotnum, "shot number"},
                  {F, &g.sx0, "first shot x"},
                  {F, &g.sxdx, "shot interval"},
                  {F, &g.sdep, "shot depth"},
                  {F, &g.rdep, "receiver depth"},
                  {F, &g.offset, "maximum offset"},
                  {F, &g.trdx, "trace interval"},
                  {F, &g.dx, "dx"},
                  {F, &g.dz, "dz"},
                  {I, &g.nx, "nx"},
                  {I, &g.nz, "nz"}},
                 err);
}

namespace {
bool write_floats(const std::string &path, const void *p, size_t size, size_t n, std::string &err) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(p, size, n, f) != n) {
        if (f) std::fclose(f);
        err = "cannot write " + path;
        return false;
    }
    std::fclose(f);
    return true;
}
}  // namespace

// Shots at sx0 + i*sxdx; receivers every trdx over [xs - offset, xs + offset]
// cut to the model.  Float arithmetic as the reference generator's.
bool write_geometry(const GeometryParams &g, const std::string &dir, std::string &err, bool verbose) {
    if (g.shotnum < 0 || g.trdx <= 0.f) {
        err = "bad geometry parameters";
        return false;
    }
    const std::string pre = dir.empty() ? std::string() : dir + "/";
    const float xmax = (float)(g.nx - 1) * g.dx, zmax = (float)(g.nz - 1) * g.dz;
    std::vector<int> tracenum(g.shotnum);
    std::vector<float> sxp(g.shotnum), szp(g.shotnum);
    for (int i = 0; i < g.shotnum; i++) {
        sxp[i] = g.sx0 + (float)i * g.sxdx;
        szp[i] = g.sdep;
        if (sxp[i] < 0.f || sxp[i] > xmax || szp[i] < 0.f || szp[i] > zmax) {
            err = "shot position exceeds model scope (shot " + std::to_string(i) + ")";
            return false;
        }
        const float lo = sxp[i] - g.offset, hi = sxp[i] + g.offset;
        const float xlp = lo > 0.f ? lo : 0.f;
        const float xrp = hi < xmax ? hi : xmax;
        const int nr = (int)((xrp - xlp) / g.trdx) + 1;
        std::vector<float> rx(nr), rz(nr, g.rdep);
        for (int j = 0; j < nr; j++) {
            rx[j] = xlp + (float)j * g.trdx;
            if (rx[j] < 0.f || rx[j] > xmax || rz[j] < 0.f || rz[j] > zmax) {
                err = "receiver position exceeds model scope (shot " + std::to_string(i) + ")";
                return false;
            }
        }
        if (!write_floats(pre + "gxp" + std::to_string(i) + ".bin", rx.data(), sizeof(float), nr, err) ||
            !write_floats(pre + "gzp" + std::to_string(i) + ".bin", rz.data(), sizeof(float), nr, err))
            return false;
        tracenum[i] = nr;
        if (verbose) std::printf("id=%d nr=%d xlp=%f xrp=%f xdis=%f\n", i, nr, xlp, xrp, xrp - xlp);
    }
    return write_floats(pre + "shotxp.bin", sxp.data(), sizeof(float), sxp.size(), err) &&
           write_floats(pre + "shotzp.bin", szp.data(), sizeof(float), szp.size(), err) &&
           write_floats(pre + "tracenum.bin", tracenum.data(), sizeof(int), tracenum.size(), err);
}

}  // namespace qpcli
