// host_abi.cpp -- C ABI over the programs' host code (include/qpstd_programs.h).
#include <cstring>
#include <string>

#include "../../include/qpstd_programs.h"
#include "programs.h"

namespace {
thread_local std::string g_err;
}

extern "C" const char *qpcli_last_error(void) { return g_err.c_str(); }

extern "C" int qpcli_read_params(int program, const char *path, double *nums, int maxn, char *strs, int strs_len) {
    if (program < 0 || program > 3 || !path) {
        g_err = "bad argument";
        return -1;
    }
    qpcli::Params par;
    const qpcli::Program p = (qpcli::Program)program;
    if (!qpcli::read_params(p, path, par, g_err)) return -1;
    int n = 0;
    std::string s;
    for (const qpcli::Field &f : qpcli::param_layout(p, par)) {
        if (f.k == qpcli::FIELD_STRING) {
            s += *static_cast<const std::string *>(f.p) + "\n";
            continue;
        }
        const double v = (f.k == qpcli::FIELD_INT) ? *static_cast<const int *>(f.p) : *static_cast<const float *>(f.p);
        if (nums && n < maxn) nums[n] = v;
        n++;
    }
    if (strs && strs_len > 0) {
        const size_t m = std::min(s.size(), (size_t)strs_len - 1);
        std::memcpy(strs, s.data(), m);
        strs[m] = '\0';
    }
    return n;
}

extern "C" int qpcli_write_geometry(const char *params_path, const char *dir) {
    qpcli::GeometryParams g;
    if (!params_path || !qpcli::read_geometry_params(params_path, g, g_err) ||
        !qpcli::write_geometry(g, dir ? dir : "", g_err, false))
        return -1;
    return 0;
}

extern "C" void qpcli_cal_bbx_bbz(int nx, int nz, const float *rho, float *bbx, float *bbz) {
    qpcli::cal_bbx_bbz(nx, nz, rho, bbx, bbz);
}
extern "C" void qpcli_rik_cal(int tmax, float dt, float fd, int flag, float *rik) {
    qpcli::rik_cal(tmax, dt, fd, flag, rik);
}
extern "C" void qpcli_transfermodel(int n, float fd, float fo, const float *vp, const float *qp, float *gam,
                                    float *lam, float *vwd, float *tao) {
    qpcli::transfermodel(n, fd, fo, vp, qp, gam, lam, vwd, tao);
}
extern "C" void qpcli_get_max_min(int n, const float *a, float *vmax, float *vmin) {
    qpcli::get_max_min(n, a, vmax, vmin);
}
extern "C" float qpcli_cfl_number(float vmax, float dt, float dx, float dz) {
    return qpcli::cfl_number(vmax, dt, dx, dz);
}
extern "C" void qpcli_distribute(int shotnum, int nranks, int rank, int *first, int *count) {
    qpcli::distribute(shotnum, nranks, rank, first, count);
}
extern "C" int qpcli_window_width(float sroffmx, float disx, float dx) {
    return qpcli::window_width(sroffmx, disx, dx);
}
