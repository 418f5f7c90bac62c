// noalloc.cu -- acoustic time steps that allocate no device memory.
//
// Some callers cannot call cudaMalloc: plug-ins that may only touch the buffers
// their host application hands them, hosts whose device memory all belongs to a
// pool they do not control, and callers on a latency-critical path where an
// allocation (and the implicit device synchronisation cudaFree brings) is not
// allowed.  For them, qpstd_ac_advance_noalloc runs the fused acoustic
// step (the same z and x pass kernels as qpstd_shot_advance) with all of its
// scratch -- the carried x divergence, div, the z part of the Laplacian, the
// per-point coefficients, the FFT and convolution tables, the CPML profiles
// and the receiver lists -- in the file-scope array g_noalloc_scratch below.
// Every GPU that loads the library holds that array (QPSTD_NOALLOC_FLOATS
// floats, 24 MiB) until the process exits.  The caller passes the model and
// the wavefield state in device memory it owns; the call copies tables into
// the array and launches kernels, nothing else.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress, so that first call should come before any stream
// capture on that device.  All calls share the one array and it keeps the
// last call's contents; every value a call reads from it is written by the same
// call first.  Calls that overlap on the GPU (different streams or threads)
// race on the array: the caller must serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qpstd.h"
#include "host_setup.h"
#include "qpstd_internal.h"

namespace qp {
void launch_ac_zpass(const AcZArgs& a, cudaStream_t s);
void launch_ac_xpass(const AcXArgs& a, cudaStream_t s);
int ac_set_smem_limits();
void set_last_error(const std::string& m);  // the message qpstd_last_error returns
}  // namespace qp

using namespace qp;

static __device__ __align__(256) float g_noalloc_scratch[QPSTD_NOALLOC_FLOATS];

namespace {

std::mutex g_mu;
float* g_addr[64] = {nullptr};  // device address of g_noalloc_scratch, per device

int fail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

__global__ void noalloc_coef_kernel(int N, float dt, const float* __restrict__ vp, const float* __restrict__ rho,
                                    float* c1, float* c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    // in double, rounded once, as qpstd_shot_create computes them on the host
    const double v = vp[i], t = dt;
    c1[i] = (float)((double)rho[i] * v * v * t);
    c2[i] = (float)(v * v * t * t / 12.0);
}

// Host image of the table region of the static array: blocks are appended at
// 64-float alignment and addressed on the device as base + offset.
struct TableImage {
    float* dev_base;      // device address of the region's first float
    size_t cap;           // floats available
    std::vector<float> h;
    float* reserve(size_t n) {
        const size_t at = (h.size() + 63) / 64 * 64;
        if (at + n > cap) return nullptr;
        h.resize(at + n, 0.f);
        return dev_base + at;
    }
    float* host_of(const float* dev) { return h.data() + (dev - dev_base); }
};

const float2* put_complex(TableImage& im, const std::vector<std::complex<double>>& v) {
    float* p = im.reserve(2 * v.size());
    if (!p) return nullptr;
    float* q = im.host_of(p);
    for (size_t i = 0; i < v.size(); i++) {
        q[2 * i] = (float)v[i].real();
        q[2 * i + 1] = (float)v[i].imag();
    }
    return reinterpret_cast<const float2*>(p);
}

const float* put_real(TableImage& im, const std::vector<double>& v) {
    float* p = im.reserve(v.size());
    if (!p) return nullptr;
    float* q = im.host_of(p);
    for (size_t i = 0; i < v.size(); i++) q[i] = (float)v[i];
    return p;
}

// Device view of a convolution plan whose twiddles live in the image:
// QPSTD_OK, QPSTD_ENOTSUP when a pass needs more threads per line than a CTA
// holds (as qpstd_shot_create reports it), QPSTD_EINVAL when the twiddles do
// not fit the static array.
int put_plan(TableImage& im, const HostPlan& hp, FFTPlanDev& pd) {
    int maxb = 1;
    for (int r : hp.rad) maxb = std::max(maxb, hp.m / r);
    if (maxb > QP_MAXTHREADS)
        return fail(QPSTD_ENOTSUP, "transform needs more threads per line than a CTA holds");
    const float2* tw = put_complex(im, hp.w);
    if (!tw) return fail(QPSTD_EINVAL, "tables exceed the static scratch");
    pd.n = hp.n;
    pd.m = hp.m;
    pd.blue = 0;
    pd.nst = (int)hp.rad.size();
    int ns = 1;
    for (int i = 0; i < pd.nst; i++) {
        FFTPass& q = pd.pass[i];
        q.R = hp.rad[i];
        q.ns = ns;
        q.B = hp.m / q.R;
        q.twstride = hp.m / (ns * q.R);
        q.ns_magic = (ns > 1) ? (unsigned)(((1ull << 32) + ns - 1) / ns) : 0u;
        ns *= q.R;
    }
    pd.tx = (maxb + 31) / 32 * 32;
    pd.w = tw;
    pd.chirp = pd.bhat = nullptr;
    return QPSTD_OK;
}

int lines_per_cta(int pairs, const FFTPlanDev& pd, size_t extra_per_line, size_t budget, bool pow2) {
    const size_t per_line = (size_t)8 * pd.m + extra_per_line;
    const int lmax = std::max(1, std::min(QP_MAXTHREADS / pd.tx, (int)(budget / per_line)));
    int L = std::max(1, std::min((pairs + 303) / 304, lmax));
    if (pow2) {
        int p = 1;
        while (p * 2 <= L) p *= 2;
        L = p;
    }
    return L;
}

}  // namespace

extern "C" int qpstd_ac_advance_noalloc(const qpstd_shot_desc* d, const float* vp, const float* rho,
                                        const float* bbx, const float* bbz, float* state, int t0, int nsteps,
                                        float* gather, void* stream) {
    if (!d || !vp || !rho || !bbx || !bbz || !state || nsteps < 0 || t0 < 0)
        return fail(QPSTD_EINVAL, "null argument or negative step index");
    if (d->kind != QPSTD_APS && d->kind != QPSTD_ARTM) return fail(QPSTD_EINVAL, "acoustic shots only");
    if (d->pml < 2 || d->nxx < 2 * d->pml + 1 || d->nzz < 2 * d->pml + 1) return fail(QPSTD_EINVAL, "bad grid");
    if (!d->rik || t0 + nsteps > d->nt) return fail(QPSTD_EINVAL, "steps beyond the source wavelet");
    if (d->xsg < 0 || d->xsg >= d->nxx || d->zsg < 0 || d->zsg >= d->nzz) return fail(QPSTD_EINVAL, "bad source");
    if (d->nr < 0 || (d->nr > 0 && (!d->gxg || !d->gzg))) return fail(QPSTD_EINVAL, "bad receivers");
    for (int i = 0; i < d->nr; i++)
        if (d->gxg[i] < 0 || d->gxg[i] >= d->nxx || d->gzg[i] < 0 || d->gzg[i] >= d->nzz)
            return fail(QPSTD_EINVAL, "receiver grid index exceeds model");
    const int nxx = d->nxx, nzz = d->nzz;
    const size_t N = (size_t)nxx * nzz;
    if (N > (size_t)QPSTD_NOALLOC_MAX_POINTS)
        return fail(QPSTD_EINVAL, "grid larger than the static scratch allows (nxx*nzz <= QPSTD_NOALLOC_MAX_POINTS)");
    if (nsteps == 0) return QPSTD_OK;
    cudaStream_t st = (cudaStream_t)stream;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(QPSTD_ECUDA, "cudaGetDevice failed");
    float* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return fail(QPSTD_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            if (ac_set_smem_limits()) return fail(QPSTD_ECUDA, "cannot raise the shared-memory limit of the pass kernels");
            g_addr[dev] = static_cast<float*>(p);
        }
        base = g_addr[dev];
    }

    // ---- layout: five N-float fields, then the table region ----
    float* Dx = base;
    float* div = base + N;
    float* Lzf = base + 2 * N;
    float* c1 = base + 3 * N;
    float* c2 = base + 4 * N;
    const size_t tab0 = (5 * N + 63) / 64 * 64;
    TableImage im{base + tab0, (size_t)QPSTD_NOALLOC_FLOATS - tab0, {}};

    HostPlan cx, cz;
    if (build_conv_plan_host(nxx, cx) || build_conv_plan_host(nzz, cz))
        return fail(QPSTD_ENOTSUP, "no convolution plan for this length");
    FFTPlanDev px{}, pz{};
    int prc = put_plan(im, cx, px);
    if (prc == QPSTD_OK) prc = put_plan(im, cz, pz);
    if (prc != QPSTD_OK) return prc;
    std::vector<std::complex<double>> H, T;
    const float2* tab[6];  // x velocity, x pressure, z velocity, z pressure derivatives; kx^2; kz^2
    for (int w = 0; w < 4; w++) {
        shift_symbols(w < 2 ? nxx : nzz, w < 2 ? d->dx : d->dz, w, H);
        conv_table(w < 2 ? cx : cz, H, T);
        tab[w] = put_complex(im, T);
    }
    for (int a = 0; a < 2; a++) {
        const int n = a ? nzz : nxx;
        const double sp = a ? d->dz : d->dx;
        H.assign(n, 0.0);
        for (int i = 0; i < n; i++) {
            const double k = wavenumber(i, n, sp);
            H[i] = k * k / n;
        }
        conv_table(a ? cz : cx, H, T);
        tab[4 + a] = put_complex(im, T);
    }
    std::vector<double> pmlv[8];  // i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz
    pml_coeffs(d->pml, d->fd, nxx, nzz, d->dx, d->dz, d->dt, pmlv);
    const float* pm[8];
    for (int k = 0; k < 8; k++) pm[k] = put_real(im, pmlv[k]);
    for (int k = 0; k < 6; k++)
        if (!tab[k]) return fail(QPSTD_EINVAL, "tables exceed the static scratch");
    for (int k = 0; k < 8; k++)
        if (!pm[k]) return fail(QPSTD_EINVAL, "tables exceed the static scratch");

    // tile shapes and staging as qpstd_shot_create chooses them
    const size_t stz = (size_t)40 * nzz, stx = (size_t)72 * nxx;
    const bool stage_z = ((size_t)8 * pz.m + stz) <= (size_t)QP_SMEM_DYN_MAX;
    const bool stage_x = ((size_t)8 * px.m + stx) <= (size_t)QP_SMEM_DYN_MAX;
    const int Lx = lines_per_cta((nzz + 1) / 2, px, stage_x ? stx : 0,
                                 stage_x ? (size_t)QP_SMEM_DYN_MAX : 160 * 1024, true);
    int Lzp = lines_per_cta((nxx + 1) / 2, pz, stage_z ? stz : 0, 110 * 1024, false);
    if (stage_z && (size_t)8 * pz.m + stz > 110 * 1024) Lzp = 1;

    // receivers grouped by x-pass tile; per cell the highest index injects
    const int TZ = 2 * Lx, ntile = (nzz + TZ - 1) / TZ;
    std::vector<std::vector<RecEntry>> per(ntile);
    for (int i = 0; i < d->nr; i++) {
        RecEntry e{d->gxg[i], d->gzg[i], i, 1};
        for (int j = i + 1; j < d->nr; j++)
            if (d->gxg[i] == d->gxg[j] && d->gzg[i] == d->gzg[j]) {
                e.inject = 0;
                break;
            }
        per[e.gz / TZ].push_back(e);
    }
    std::vector<int> roff(ntile + 1, 0);
    std::vector<RecEntry> flat;
    for (int t = 0; t < ntile; t++) {
        roff[t] = (int)flat.size();
        flat.insert(flat.end(), per[t].begin(), per[t].end());
    }
    roff[ntile] = (int)flat.size();
    float* roff_d = im.reserve(roff.size());
    float* rec_d = im.reserve(4 * std::max<size_t>(flat.size(), 1));
    if (!roff_d || !rec_d) return fail(QPSTD_EINVAL, "receivers exceed the static scratch");
    memcpy(im.host_of(roff_d), roff.data(), sizeof(int) * roff.size());
    if (!flat.empty()) memcpy(im.host_of(rec_d), flat.data(), sizeof(RecEntry) * flat.size());

    // ---- device work: table upload, coefficients, the pipelined steps ----
    cudaError_t e = cudaMemcpyAsync(base + tab0, im.h.data(), sizeof(float) * im.h.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(QPSTD_ECUDA, std::string("table upload: ") + cudaGetErrorString(e));
    noalloc_coef_kernel<<<(unsigned)((N + 255) / 256), 256, 0, st>>>((int)N, d->dt, vp, rho, c1, c2);

    float* p = state;
    float *vx = state + N, *vz = state + 2 * N, *fipx = state + 3 * N, *fipz = state + 4 * N;
    float *fivxx = state + 5 * N, *fivzz = state + 6 * N;
    auto zargs = [&](int do_v, int do_div) {
        AcZArgs a{};
        a.nxx = nxx; a.nzz = nzz; a.L = Lzp; a.pl = pz;
        a.HzM = tab[2]; a.HzP = tab[3]; a.kz2 = tab[5];
        a.i_az = pm[2]; a.i_bz = pm[3]; a.h_az = pm[6]; a.h_bz = pm[7];
        a.bbz = bbz; a.p = p; a.vz = vz; a.psi_pz = fipz; a.psi_vz = fivzz; a.Dx = Dx;
        a.div = div; a.Lz = Lzf; a.dt = d->dt; a.do_v = do_v; a.do_div = do_div; a.stage = stage_z;
        return a;
    };
    auto xargs = [&](int do_p, int do_v, int do_dx) {
        AcXArgs a{};
        a.nxx = nxx; a.nzz = nzz; a.L = Lx; a.pml = d->pml; a.pl = px;
        a.HxM = tab[0]; a.HxP = tab[1]; a.kx2 = tab[4];
        a.i_ax = pm[0]; a.i_bx = pm[1]; a.h_ax = pm[4]; a.h_bx = pm[5];
        a.bbx = bbx; a.c1 = c1; a.c2 = c2; a.p = p; a.vx = vx; a.psi_px = fipx; a.psi_vx = fivxx; a.Dx = Dx;
        a.div = div; a.Lz = Lzf; a.dt = d->dt; a.do_p = do_p; a.do_v = do_v; a.do_dx = do_dx;
        a.xs = -1; a.zs = -1; a.stage = stage_x;
        return a;
    };
    launch_ac_xpass(xargs(0, 0, 1), st);
    for (int t = t0; t < t0 + nsteps; t++) {
        launch_ac_zpass(zargs(t > t0, 1), st);
        AcXArgs x = xargs(1, 1, t < t0 + nsteps - 1);
        x.xs = d->xsg;
        x.zs = d->zsg;
        x.src = (float)((double)d->rik[t] * d->dt * 1000.0);
        x.rec_off = reinterpret_cast<const int*>(roff_d);
        x.rec = reinterpret_cast<const RecEntry*>(rec_d);
        x.gather_row = (gather && d->nr > 0) ? gather + (size_t)(t - t0) * d->nr : nullptr;
        launch_ac_xpass(x, st);
    }
    launch_ac_zpass(zargs(1, 0), st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QPSTD_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return QPSTD_OK;
}
