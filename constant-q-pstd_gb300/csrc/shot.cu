// shot.cu -- per-shot device state, the step schedule and the C ABI.
//
// One shot owns one stream, its windowed model and coefficient tables, the
// source wavefield and (RTM) the receiver wavefield, the revolve checkpoint
// pool and the image accumulators, all resident in HBM.  The reference's
// per-shot body of acforward (e.g. sgpstd-qrtm/acsglw.cu:304-1079) maps onto
// qpstd_shot_create + qpstd_shot_rtm_device + qpstd_shot_get_image.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qpstd.h"
#include "host_setup.h"
#include "qpstd_internal.h"
#include "revolve.h"
#include "shot.h"

namespace qp {
void launch_ac_zpass(const AcZArgs& a, cudaStream_t s);
void launch_ac_xpass(const AcXArgs& a, cudaStream_t s);
int ac_set_smem_limits();
void launch_vz_passA(const VzArgsA& a, cudaStream_t s);
void launch_vz_xspec(const VxsArgs& a, cudaStream_t s);
void launch_vz_passB(const VzArgsB& a, cudaStream_t s);
void launch_vz_passC(const VzArgsC& a, cudaStream_t s);
void launch_vz_zinv(const VzArgsI& a, cudaStream_t s);
void launch_vz_xspec_conv(const VxsArgs& a, cudaStream_t s);
void launch_vz_convtab(const VtabArgs& a, cudaStream_t s);
void launch_lr_xconv(const LrxArgs& a, cudaStream_t s);
void launch_lr_zsum(const LrsArgs& a, cudaStream_t s);
int vz_set_smem_limits();
}  // namespace qp

using namespace qp;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
static int cuda_fail(cudaError_t e, const char* where) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? QPSTD_ENOMEM : QPSTD_ECUDA;
}
#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
    } while (0)

extern "C" const char* qpstd_last_error(void) { return g_err.c_str(); }

// Shared-memory bytes per line pair that the x pass stages, for its largest
// mode in a shot of this kind: the acoustic step (p update, v, next Dx) or the
// constant-Q step (v, next Dx).
static size_t xstage_bytes(bool visco, int nxx) {
    const unsigned f = visco ? qp::xstage_fields(0, 1, 1) : qp::xstage_fields(1, 1, 1);
    return (size_t)8 * qp::xstage_count(f) * nxx;
}

namespace qp {
void set_last_error(const std::string& m) { g_err = m; }
}  // namespace qp
extern "C" int qpstd_version(void) { return 100; }

// ---------------------------------------------------------------------------
__global__ void add_point_kernel(float* p, float v) { p[0] += v; }

// Every device buffer of a shot: from its arena when it has one (shots of a
// server), else cudaMalloc; recorded for release at destroy.
cudaError_t shot_malloc(qpstd_shot* s, void** p, size_t bytes) {
    if (s->arena) {
        *p = s->arena->alloc(bytes);
        if (!*p) return cudaErrorMemoryAllocation;
    } else {
        const cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) return e;
    }
    s->allocs.push_back(*p);
    return cudaSuccess;
}

static int upload_plan(qpstd_shot* s, const HostPlan& hp, FFTPlanDev& d) {
    if (fill_plan_dev(hp, d)) return fail(QPSTD_ENOTSUP, "transform needs more threads per line than a CTA holds");
    std::vector<float2> h;
    plan_tables(hp, h);
    const size_t cnt = h.size();
    float2* dptr = nullptr;
    CK(shot_malloc(s, (void**)&dptr, sizeof(float2) * cnt));
    CK(cudaMemcpy(dptr, h.data(), sizeof(float2) * cnt, cudaMemcpyHostToDevice));
    d.w = dptr;
    d.chirp = hp.blue ? dptr + hp.w.size() : nullptr;
    d.bhat = hp.blue ? dptr + hp.w.size() + hp.chirp.size() : nullptr;
    return QPSTD_OK;
}

static int validate(const qpstd_shot_desc* d) {
    if (!d) return fail(QPSTD_EINVAL, "null descriptor");
    if (d->kind < QPSTD_APS || d->kind > QPSTD_QRTM) return fail(QPSTD_EINVAL, "bad kind");
    if (d->pml < 2 || d->nxx < 2 * d->pml + 1 || d->nzz < 2 * d->pml + 1)
        return fail(QPSTD_EINVAL, "grid smaller than twice the CPML width");
    if (d->nt < 1) return fail(QPSTD_EINVAL, "nt < 1");
    if (!d->vp || !d->rho || !d->bbx || !d->bbz || !d->rik) return fail(QPSTD_EINVAL, "null model pointer");
    const bool visco = d->kind == QPSTD_VAPS || d->kind == QPSTD_QRTM;
    if (visco && (!d->gam || !d->lam || !d->vwd || !d->tao)) return fail(QPSTD_EINVAL, "null Q model pointer");
    if (d->xsg < 0 || d->xsg >= d->nxx || d->zsg < 0 || d->zsg >= d->nzz)
        return fail(QPSTD_EINVAL, "shot grid index exceeds model");
    if (d->nr < 0 || (d->nr > 0 && (!d->gxg || !d->gzg))) return fail(QPSTD_EINVAL, "bad receivers");
    for (int i = 0; i < d->nr; i++)
        if (d->gxg[i] < 0 || d->gxg[i] >= d->nxx || d->gzg[i] < 0 || d->gzg[i] >= d->nzz)
            return fail(QPSTD_EINVAL, "receiver grid index exceeds model");
    const bool rtm = d->kind == QPSTD_ARTM || d->kind == QPSTD_QRTM;
    if (rtm && (d->snaps < 1 || d->snaps > 64)) return fail(QPSTD_EINVAL, "snaps must be in 1..64");
    if (d->method != QPSTD_FUSED && d->method != QPSTD_PLAIN) return fail(QPSTD_EINVAL, "bad method");
    return QPSTD_OK;
}

static float* dalloc(qpstd_shot* s, size_t n, int* rc) {
    float* p = nullptr;
    cudaError_t e = shot_malloc(s, (void**)&p, sizeof(float) * n);
    if (e != cudaSuccess) {
        *rc = cuda_fail(e, "cudaMalloc");
        return nullptr;
    }
    return p;
}

// Receivers grouped by the CTA tile that owns their cell: x passes tile the z
// axis (key gz / width), z passes tile the x axis (key gx / width).
static int build_rec_list(qpstd_shot* s, const qpstd_shot_desc* d, int width, bool key_x, int** off_out,
                          RecEntry** rec_out) {
    const int ntile = ((key_x ? d->nxx : d->nzz) + width - 1) / width;
    std::vector<std::vector<RecEntry>> per(ntile);
    // winning receiver per cell: the reference marks flagrec/rindex per cell,
    // the last receiver written wins (acsglw.cu:387-403)
    std::vector<int> win(d->nr, 1);
    for (int i = 0; i < d->nr; i++)
        for (int j = i + 1; j < d->nr; j++)
            if (d->gxg[i] == d->gxg[j] && d->gzg[i] == d->gzg[j]) {
                win[i] = 0;
                break;
            }
    for (int i = 0; i < d->nr; i++) {
        RecEntry e;
        e.gx = d->gxg[i];
        e.gz = d->gzg[i];
        e.ir = i;
        e.inject = win[i];
        per[(key_x ? e.gx : e.gz) / width].push_back(e);
    }
    std::vector<int> off(ntile + 1, 0);
    std::vector<RecEntry> flat;
    for (int t = 0; t < ntile; t++) {
        off[t] = (int)flat.size();
        flat.insert(flat.end(), per[t].begin(), per[t].end());
    }
    off[ntile] = (int)flat.size();
    int* doff = nullptr;
    CK(shot_malloc(s, (void**)&doff, sizeof(int) * off.size()));
    CK(cudaMemcpy(doff, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
    RecEntry* drec = nullptr;
    const size_t nrec = std::max<size_t>(flat.size(), 1);
    CK(shot_malloc(s, (void**)&drec, sizeof(RecEntry) * nrec));
    if (!flat.empty()) CK(cudaMemcpy(drec, flat.data(), sizeof(RecEntry) * flat.size(), cudaMemcpyHostToDevice));
    *off_out = doff;
    *rec_out = drec;
    return QPSTD_OK;
}

static int build_receivers(qpstd_shot* s, const qpstd_shot_desc* d) {
    int rc = build_rec_list(s, d, 2 * s->Lx, false, &s->rec_off, &s->rec);
    if (rc || !s->visco) return rc;
    return build_rec_list(s, d, 2 * s->Lzv, true, &s->rec_off_z, &s->rec_z);
}

// Per-point constant-Q coefficients and the spectra scratch (double -> float once).
static int setup_visco(qpstd_shot* s, const qpstd_shot_desc* d) {
    const size_t N = s->N;
    int rc = QPSTD_OK;
    const size_t NS = (size_t)d->nxx * s->nzh;  // half-spectrum length (complex)
    float* f = dalloc(s, 8 * N, &rc);
    if (!f) return rc;
    s->y1 = f; s->y2 = f + N; s->y3c = f + 2 * N; s->y4c = f + 3 * N;
    s->e1 = f + 4 * N; s->e2 = f + 5 * N; s->e3 = f + 6 * N; s->total = f + 7 * N;
    float* sp = dalloc(s, 2 * NS * (s->rtm ? 6 : 5), &rc);
    if (!sp) return rc;
    for (int k = 0; k < 4; k++) s->spec[k] = reinterpret_cast<float2*>(sp) + k * NS;
    s->src.aux_spec = reinterpret_cast<float2*>(sp) + 4 * NS;
    if (s->rtm) s->rcv.aux_spec = reinterpret_cast<float2*>(sp) + 5 * NS;
    std::vector<float> h(7 * N);
    const double dt = d->dt;
    for (size_t i = 0; i < N; i++) {
        const double g = d->gam[i], w = d->vwd[i], vp = d->vp[i], lam = d->lam[i], tao = d->tao[i];
        const double cc = dt * dt * vp * vp * lam / 12.0;  // sum_total, acsglw.cu:1213-1245
        h[i] = (float)(1.0 - 32.0 * g);
        h[N + i] = (float)(32.0 * g * w);
        h[2 * N + i] = (float)((1.0 - 64.0 * g) * cc);
        h[3 * N + i] = (float)(64.0 * g * w * cc);
        h[4 * N + i] = (float)((double)d->rho[i] * vp * vp * dt * lam);  // addsa_kernel, acsglw.cu:1527
        h[5 * N + i] = (float)(0.5 * dt * tao);
        h[6 * N + i] = (float)(dt * tao);
    }
    CK(cudaMemcpy(f, h.data(), sizeof(float) * 7 * N, cudaMemcpyHostToDevice));
    return QPSTD_OK;
}

// Squared wavenumbers kkx^2, kkz^2 (the 2-D symbols are built from them on the fly).
static int setup_ksq(qpstd_shot* s, const qpstd_shot_desc* d) {
    int rc = QPSTD_OK;
    std::vector<float> k2(d->nxx + d->nzz);
    for (int i = 0; i < d->nxx; i++) {
        const double k = wavenumber(i, d->nxx, d->dx);
        k2[i] = (float)(k * k);
    }
    for (int j = 0; j < d->nzz; j++) {
        const double k = wavenumber(j, d->nzz, d->dz);
        k2[d->nxx + j] = (float)(k * k);
    }
    float* kk = dalloc(s, k2.size(), &rc);
    if (!kk) return rc;
    CK(cudaMemcpy(kk, k2.data(), sizeof(float) * k2.size(), cudaMemcpyHostToDevice));
    s->kxsq = kk;
    s->kzsq = kk + d->nxx;
    return QPSTD_OK;
}

// Convolution tables of the stationary constant-Q symbols.  When nxx is not a
// smooth length the exact x transforms of the x-spectral passes go through
// Bluestein (two FFTs each); a symbol that does not change in time is instead
// applied per kz column as a circular convolution along x on the smooth
// convolution length (one FFT per output after a shared forward FFT).
static int setup_xtabs(qpstd_shot* s, const qpstd_shot_desc* d) {
    if (!s->px.blue) return QPSTD_OK;
    int rc = QPSTD_OK;
    const int mc = s->pxc.m, nzh = s->nzh, mh = mc / 2 + 1;  // rows keep the even half
    float* t = dalloc(s, (size_t)4 * nzh * mh, &rc);
    if (!t) return rc;
    VtabArgs a{};
    a.nxx = d->nxx; a.nzz = d->nzz; a.nzh = nzh;
    a.pl = s->px; a.plc = s->pxc; a.kx2 = s->kxsq; a.kz2 = s->kzsq;
    a.norm = (float)(1.0 / ((double)d->nxx * d->nzz));
    a.L = choose_L(nzh, std::max(s->px.m, mc), std::max(s->px.tx, s->pxc.tx), 1, false);
    for (int k = 0; k < 4; k++) {
        a.sym = k;
        a.out = t + (size_t)k * nzh * mh;
        s->xtab[k] = a.out;
        launch_vz_convtab(a, s->stream);
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "convolution tables");
    s->xconv = true;
    s->Lxs_exact = s->Lxs;
    s->Lxs = choose_L(nzh, mc, s->pxc.tx, 1, true);
    s->Lxs3 = choose_L(nzh, mc, s->pxc.tx, 2, true);
    return QPSTD_OK;
}

// Plain form: cuFFT plan, scratch, and the reference's own shift symbols.
static int setup_plain(qpstd_shot* s, const qpstd_shot_desc* d) {
    std::string err;
    if (plain_setup(s, err)) return fail(QPSTD_ECUDA, err);
    const int lens[4] = {d->nxx, d->nxx, d->nzz, d->nzz};
    const double sp[4] = {d->dx, d->dx, d->dz, d->dz};
    const size_t nc = 2 * (size_t)d->nxx + 2 * d->nzz;
    std::vector<float2> hc(nc);
    float2* cbase = nullptr;
    CK(shot_malloc(s, (void**)&cbase, sizeof(float2) * nc));
    const float2** dst[4] = {&s->plain.HxM, &s->plain.HxP, &s->plain.HzM, &s->plain.HzP};
    size_t q = 0;
    std::vector<std::complex<double>> H;
    for (int w = 0; w < 4; w++) {
        shift_symbols(lens[w], sp[w], w, H, true);
        *dst[w] = cbase + q;
        for (auto& c : H) hc[q++] = make_float2((float)c.real(), (float)c.imag());
    }
    CK(cudaMemcpy(cbase, hc.data(), sizeof(float2) * nc, cudaMemcpyHostToDevice));
    return QPSTD_OK;
}

// Convolution plans along x and z and the length-m multipliers of the six
// separable operators (two staggered derivatives and the k^2 term per axis).
static int setup_conv(qpstd_shot* s, const qpstd_shot_desc* d) {
    HostPlan cx, cz;
    if (build_conv_plan_host(d->nxx, cx, true) || build_conv_plan_host(d->nzz, cz))
        return fail(QPSTD_ENOTSUP, "no convolution plan for this length");
    int rc;
    if ((rc = upload_plan(s, cx, s->pxc))) return rc;
    if ((rc = upload_plan(s, cz, s->pzc))) return rc;
    const size_t nc = 3 * (size_t)cx.m + 3 * (size_t)cz.m;
    std::vector<float2> hc(nc);
    float2* base = nullptr;
    CK(shot_malloc(s, (void**)&base, sizeof(float2) * nc));
    size_t q = 0;
    std::vector<std::complex<double>> H, T;
    auto put = [&](const HostPlan& hp, const std::vector<std::complex<double>>& sym, const float2** dst) {
        conv_table(hp, sym, T);
        *dst = base + q;
        for (auto& c : T) hc[q++] = make_float2((float)c.real(), (float)c.imag());
    };
    shift_symbols(d->nxx, d->dx, 0, H);
    put(cx, H, &s->cHxM);
    shift_symbols(d->nxx, d->dx, 1, H);
    put(cx, H, &s->cHxP);
    H.assign(d->nxx, 0.0);
    for (int i = 0; i < d->nxx; i++) {
        const double k = wavenumber(i, d->nxx, d->dx);
        H[i] = k * k / d->nxx;
    }
    put(cx, H, &s->cKx2);
    shift_symbols(d->nzz, d->dz, 2, H);
    put(cz, H, &s->cHzM);
    shift_symbols(d->nzz, d->dz, 3, H);
    put(cz, H, &s->cHzP);
    H.assign(d->nzz, 0.0);
    for (int j = 0; j < d->nzz; j++) {
        const double k = wavenumber(j, d->nzz, d->dz);
        H[j] = k * k / d->nzz;
    }
    put(cz, H, &s->cKz2);
    CK(cudaMemcpy(base, hc.data(), sizeof(float2) * nc, cudaMemcpyHostToDevice));
    return QPSTD_OK;
}

static int autotune(qpstd_shot* s);

extern "C" int qpstd_shot_create(const qpstd_shot_desc* d, qpstd_shot** out) {
    return shot_create_ex(d, out, true, nullptr);
}

int shot_create_ex(const qpstd_shot_desc* d, qpstd_shot** out, bool tune, qp::Arena* arena) {
    if (!out) return fail(QPSTD_EINVAL, "null output handle");
    *out = nullptr;
    int rc = validate(d);
    if (rc) return rc;
    qpstd_shot* s = new qpstd_shot();
    s->d = *d;
    s->arena = arena;
    const int nxx = d->nxx, nzz = d->nzz;
    const size_t N = (size_t)nxx * nzz;
    s->N = N;
    s->nx = nxx - 2 * d->pml;
    s->nz = nzz - 2 * d->pml;
    s->visco = (d->kind == QPSTD_VAPS || d->kind == QPSTD_QRTM);
    s->rtm = (d->kind == QPSTD_ARTM || d->kind == QPSTD_QRTM);
    s->rik.assign(d->rik, d->rik + d->nt);
    auto bail = [&](int code) {
        qpstd_shot_destroy(s);
        return code;
    };
    // the kernels' shared-memory limits are attributes of each device's context:
    // raised once per device (the current one), under a lock
    {
        static std::mutex mu;
        static bool raised[64] = {false};
        int dev = 0;
        cudaError_t de = cudaGetDevice(&dev);
        if (de != cudaSuccess) return bail(cuda_fail(de, "cudaGetDevice"));
        if (dev < 0 || dev >= 64) return bail(fail(QPSTD_ENOTSUP, "device index above 63"));
        std::lock_guard<std::mutex> lk(mu);
        if (!raised[dev]) {
            if (ac_set_smem_limits() || vz_set_smem_limits())
                return bail(fail(QPSTD_ECUDA, "cannot raise the shared-memory limit of the pass kernels"));
            raised[dev] = true;
        }
    }
    s->nzh = nzz / 2 + 1;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));

    // wavefields: 8 state fields + the pipelined Dx, contiguous
    s->src.st = dalloc(s, 9 * N, &rc);
    if (!s->src.st) return bail(rc);
    if (s->rtm) {
        s->rcv.st = dalloc(s, 9 * N, &rc);
        if (!s->rcv.st) return bail(rc);
    }
    s->div = dalloc(s, N, &rc);
    s->Lz = dalloc(s, N, &rc);
    s->bbx = dalloc(s, N, &rc);
    s->bbz = dalloc(s, N, &rc);
    s->c1 = dalloc(s, N, &rc);
    s->c2 = dalloc(s, N, &rc);
    if (!s->div || !s->Lz || !s->bbx || !s->bbz || !s->c1 || !s->c2) return bail(rc);

    // models and per-point coefficients (double -> float once)
    {
        std::vector<float> c1(N), c2(N);
        const double dt = d->dt;
        for (size_t i = 0; i < N; i++) {
            const double vp = d->vp[i];
            c1[i] = (float)((double)d->rho[i] * vp * vp * dt);
            c2[i] = (float)(vp * vp * dt * dt / 12.0);
        }
        if ((e = cudaMemcpy(s->c1, c1.data(), 4 * N, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
        if ((e = cudaMemcpy(s->c2, c2.data(), 4 * N, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
        if ((e = cudaMemcpy(s->bbx, d->bbx, 4 * N, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
        if ((e = cudaMemcpy(s->bbz, d->bbz, 4 * N, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
    }
    // 1-D tables
    {
        std::vector<double> pmlv[8];
        pml_coeffs(d->pml, d->fd, nxx, nzz, d->dx, d->dz, d->dt, pmlv);
        const size_t nt1 = 4 * (size_t)nxx + 4 * nzz + nxx + nzz;
        std::vector<float> h(nt1);
        size_t o = 0;
        float* base = dalloc(s, nt1, &rc);
        if (!base) return bail(rc);
        const float** dst[8] = {&s->i_ax, &s->i_bx, &s->i_az, &s->i_bz, &s->h_ax, &s->h_bx, &s->h_az, &s->h_bz};
        for (int k = 0; k < 8; k++) {
            *dst[k] = base + o;
            for (double v : pmlv[k]) h[o++] = (float)v;
        }
        s->kx2 = base + o;
        for (int i = 0; i < nxx; i++) {
            const double k = wavenumber(i, nxx, d->dx);
            h[o++] = (float)(k * k / nxx);
        }
        s->kz2 = base + o;
        for (int j = 0; j < nzz; j++) {
            const double k = wavenumber(j, nzz, d->dz);
            h[o++] = (float)(k * k / nzz);
        }
        if ((e = cudaMemcpy(base, h.data(), 4 * nt1, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
        std::vector<std::complex<double>> H;
        const size_t nc = 2 * (size_t)nxx + 2 * nzz;
        std::vector<float2> hc(nc);
        float2* cbase = nullptr;
        if ((e = shot_malloc(s, (void**)&cbase, sizeof(float2) * nc)) != cudaSuccess)
            return bail(cuda_fail(e, "cudaMalloc"));
        size_t q = 0;
        const float2** cdst[4] = {&s->HxM, &s->HxP, &s->HzM, &s->HzP};
        const int lens[4] = {nxx, nxx, nzz, nzz};
        const double sp[4] = {d->dx, d->dx, d->dz, d->dz};
        for (int w = 0; w < 4; w++) {
            shift_symbols(lens[w], sp[w], w, H);
            *cdst[w] = cbase + q;
            for (auto& c : H) hc[q++] = make_float2((float)c.real(), (float)c.imag());
        }
        if ((e = cudaMemcpy(cbase, hc.data(), sizeof(float2) * nc, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(cuda_fail(e, "upload"));
    }
    // FFT plans and tile shapes of the fused passes (the plain form uses cuFFT)
    if (d->method == QPSTD_FUSED) {
        HostPlan hx, hz;
        if (build_plan_host(nxx, hx, true) || build_plan_host(nzz, hz))
            return bail(fail(QPSTD_ENOTSUP, "no FFT plan for this length"));
        if ((rc = upload_plan(s, hx, s->px))) return bail(rc);
        if ((rc = upload_plan(s, hz, s->pz))) return bail(rc);
        if ((rc = setup_conv(s, d))) return bail(rc);
        const int pairs_z = (nxx + 1) / 2, pairs_x = (nzz + 1) / 2;
        // acoustic passes: stage the epilogue inputs when they fit beside the lines
        // (z: 5 fields x 2 rows x nzz floats per line; x: up to 9 fields x 2 columns x nxx)
        const size_t stz = (size_t)40 * nzz, stx = xstage_bytes(s->visco, nxx);
        s->stage_z = ((size_t)8 * s->pzc.m + stz) <= (size_t)QP_SMEM_DYN_MAX;
        s->stage_x = ((size_t)8 * s->pxc.m + stx) <= (size_t)QP_SMEM_DYN_MAX;
        s->Lx = choose_L(pairs_x, s->pxc.m, s->pxc.tx, 1, true, s->stage_x ? stx : 0,
                         s->stage_x ? (size_t)QP_SMEM_DYN_MAX : 160 * 1024);
        s->Lzp = choose_L(pairs_z, s->pzc.m, s->pzc.tx, 1, false, s->stage_z ? stz : 0, 110 * 1024);
        if (s->stage_z && (size_t)8 * s->pzc.m + stz > 110 * 1024) s->Lzp = 1;
        // constant-Q: z pass B and the 3-output x-spectral pass hold two line buffers;
        // z pass A uses both the exact and the convolution plan
        s->Lzv = choose_L(pairs_z, std::max(s->pz.m, s->pzc.m), std::max(s->pz.tx, s->pzc.tx), 2, false);
        s->Lxs = choose_L(s->nzh, s->px.m, s->px.tx, 1, true);
        s->Lxs3 = choose_L(s->nzh, s->px.m, s->px.tx, 2, true);
        const int mmax = std::max(std::max(s->px.m, s->pz.m), std::max(s->pxc.m, s->pzc.m));
        if (16.0 * mmax > 200 * 1024) return bail(fail(QPSTD_ENOTSUP, "line too long for one CTA"));
    }
    if (s->visco && (rc = setup_visco(s, d))) return bail(rc);
    if ((rc = setup_ksq(s, d))) return bail(rc);
    if (s->visco && d->method == QPSTD_FUSED && (rc = setup_xtabs(s, d))) return bail(rc);
    if (d->method == QPSTD_PLAIN && (rc = setup_plain(s, d))) return bail(rc);
    s->gather = dalloc(s, (size_t)d->nt * std::max(d->nr, 1), &rc);
    if (!s->gather) return bail(rc);
    if (s->rtm) {
        s->store = dalloc(s, (size_t)d->snaps * 8 * N, &rc);
        s->obs = dalloc(s, (size_t)d->nt * std::max(d->nr, 1), &rc);
        s->img = dalloc(s, 4 * (size_t)s->nx * s->nz, &rc);
        if (!s->store || !s->obs || !s->img) return bail(rc);
        s->img_c = s->img + (size_t)s->nx * s->nz;
        s->ssg = s->img_c + (size_t)s->nx * s->nz;
        s->ssg_c = s->ssg + (size_t)s->nx * s->nz;
    }
    // the receiver lists are grouped by the CTA tiles (x pass: 2*Lx z columns,
    // z pass C: 2*Lzv x rows), so they are built once the tile sizes are final
    if (tune && (rc = autotune(s))) return bail(rc);
    if ((rc = build_receivers(s, d))) return bail(rc);
    s->src.aux_pending = false;
    if ((e = cudaMemset(s->src.st, 0, sizeof(float) * 9 * N)) != cudaSuccess) return bail(cuda_fail(e, "memset"));
    *out = s;
    return QPSTD_OK;
}

extern "C" int qpstd_shot_destroy(qpstd_shot* s) {
    if (!s) return QPSTD_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto& t : s->timed) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    for (cudaEvent_t e : s->evpool) cudaEventDestroy(e);
    plain_release(s);
    for (void* p : s->allocs) {
        if (s->arena) s->arena->release(p);
        else cudaFree(p);
    }
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return QPSTD_OK;
}

extern "C" int qpstd_shot_set_state(qpstd_shot* s, const float* state) {
    if (!s || !state) return fail(QPSTD_EINVAL, "null argument");
    CK(cudaMemcpyAsync(s->src.st, state, sizeof(float) * 8 * s->N, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->src.aux_pending = false;
    return QPSTD_OK;
}

extern "C" int qpstd_shot_get_state(qpstd_shot* s, float* state) {
    if (!s || !state) return fail(QPSTD_EINVAL, "null argument");
    CK(cudaMemcpyAsync(state, s->src.st, sizeof(float) * 8 * s->N, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return QPSTD_OK;
}

// ---------------------------------------------------------------------------
// per-launch timing
static cudaEvent_t pool_event(qpstd_shot* s) {
    if (!s->evpool.empty()) {
        cudaEvent_t e = s->evpool.back();
        s->evpool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
struct ProfScope {
    qpstd_shot* s;
    int kind;
    cudaEvent_t a = nullptr;
    ProfScope(qpstd_shot* s_, int k, int count = 1) : s(s_), kind(k) {
        if (s->prof) {
            a = pool_event(s);
            cudaEventRecord(a, s->stream);
        }
        s->launches += count;
    }
    ~ProfScope() {
        if (s->prof) {
            cudaEvent_t b = pool_event(s);
            cudaEventRecord(b, s->stream);
            s->timed.push_back({kind, a, b});
        }
    }
};

// ---------------------------------------------------------------------------
// acoustic passes
static AcZArgs zargs(qpstd_shot* s, Wave& w, int do_v, int do_div) {
    AcZArgs a;
    a.nxx = s->d.nxx;
    a.nzz = s->d.nzz;
    a.L = s->Lzp;
    a.pl = s->pzc;
    a.HzP = s->cHzP;
    a.HzM = s->cHzM;
    a.kz2 = s->cKz2;
    a.h_az = s->h_az;
    a.h_bz = s->h_bz;
    a.i_az = s->i_az;
    a.i_bz = s->i_bz;
    a.bbz = s->bbz;
    a.p = w.p(s->N);
    a.vz = w.vz(s->N);
    a.psi_pz = w.fipz(s->N);
    a.psi_vz = w.fivzz(s->N);
    a.Dx = w.Dx(s->N);
    a.div = s->div;
    a.Lz = s->Lz;
    a.dt = s->d.dt;
    a.do_v = do_v;
    a.do_div = do_div;
    a.stage = s->stage_z ? 1 : 0;
    return a;
}

static AcXArgs xargs(qpstd_shot* s, Wave& w, int do_p, int do_v, int do_dx) {
    AcXArgs a;
    memset(&a, 0, sizeof(a));
    a.nxx = s->d.nxx;
    a.nzz = s->d.nzz;
    a.L = s->Lx;
    a.pml = s->d.pml;
    a.pl = s->pxc;
    a.HxP = s->cHxP;
    a.HxM = s->cHxM;
    a.kx2 = s->cKx2;
    a.h_ax = s->h_ax;
    a.h_bx = s->h_bx;
    a.i_ax = s->i_ax;
    a.i_bx = s->i_bx;
    a.bbx = s->bbx;
    a.c1 = s->c1;
    a.c2 = s->c2;
    a.p = w.p(s->N);
    a.vx = w.vx(s->N);
    a.psi_px = w.fipx(s->N);
    a.psi_vx = w.fivxx(s->N);
    a.Dx = w.Dx(s->N);
    a.div = s->div;
    a.Lz = s->Lz;
    a.dt = s->d.dt;
    a.do_p = do_p;
    a.do_v = do_v;
    a.do_dx = do_dx;
    a.xs = -1;
    a.zs = -1;
    a.stage = s->stage_x ? 1 : 0;
    return a;
}

// The source wavefield runs as a pipeline: begin() computes the x part of the
// first step's divergence, each step() is one z pass and one x pass (the x
// pass also prepares the next step's x divergence unless it is the last), and
// end() applies the last step's pending z-velocity update.  Between end() and
// the next begin() the eight state fields are exactly the reference's state.
static void src_begin(qpstd_shot* s) {
    if (s->d.method == QPSTD_PLAIN) return;  // the plain form keeps no state between steps
    ProfScope ps(s, QPSTD_K_XPASS);
    launch_ac_xpass(xargs(s, s->src, 0, 0, 1), s->stream);
}

// One plain-form step (all of its cuFFT calls and kernels timed as one unit).
static void plain_one(qpstd_shot* s, Wave& w, float src, int t_filter, float eta, float* gather_row,
                      const float* obs_row, bool ssg_on, bool image) {
    ProfScope ps(s, QPSTD_K_PLAIN, 0);
    const int rc = plain_step(s, w, src, t_filter, eta, gather_row, obs_row, ssg_on, image, &s->launches);
    if (rc && !s->plain_err) s->plain_err = rc;
}

// The Q-RTM stabilised symbol S = ka - 2 eta ka (1 + tau dt ka) / (exp(-tau tt ka)
// + eta exp(tau dt ka)) (multt_kernel, sgpstd-qrtm/acsglw.cu:1895, float
// arithmetic, tt = t dt) rounds to ka itself while its correction stays below a
// quarter ulp of ka, which with the reference's eta ~ 1e-26 holds for every
// step of ordinary runs.  The correction grows with tt, so per eta the largest
// such step is found once (over 4096 samples of ka up to the grid's largest);
// steps up to it use the k^1.01 operator -- the per-kz convolution when the
// width needs Bluestein -- instead of exact transforms.
static bool filter_is_ka(qpstd_shot* s, float eta, int t) {
    for (auto& c : s->ka_steps)
        if (c.first == eta) return t <= c.second;
    const double kx = wavenumber(s->d.nxx / 2, s->d.nxx, s->d.dx), kz = wavenumber(s->d.nzz / 2, s->d.nzz, s->d.dz);
    const double kmax2 = kx * kx + kz * kz;  // the largest |k|^2 of the grid
    const double e6 = (double)eta * 1e-6, tau = s->d.taoc, dt = s->d.dt;
    auto plain_at = [&](int tt_idx) {
        const double tt = (double)tt_idx * dt;
        for (int i = 1; i <= 4096; i++) {
            const double ka = std::pow(kmax2 * i / 4096.0, 0.505);
            const double corr = 2.0 * e6 * (1.0 + tau * dt * ka) / (std::exp(-tau * tt * ka) + e6 * std::exp(tau * dt * ka));
            if (!(corr < std::ldexp(1.0, -26))) return false;
        }
        return true;
    };
    int lo = -1, hi = s->d.nt;  // plain_at(lo) holds (or lo = -1), plain_at(hi) is never asked
    if (plain_at(s->d.nt)) lo = s->d.nt;
    else
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (plain_at(mid)) lo = mid;
            else hi = mid;
        }
    s->ka_steps.push_back({eta, lo});
    return t <= lo;
}

// One constant-Q step of wavefield w (seven launches, see vz_kernels.cu).
// src: amplitude at the source this step; t_filter / eta: time index and
// stabilisation of the Q-RTM aux filter; last: skip the next step's Dx;
// gather_row / obs_row / ssg_on / image: receiver recording, Dirichlet
// injection, illumination and imaging, all inside z pass C.
static void vz_step(qpstd_shot* s, Wave& w, float src, int t_filter, float eta, bool last, float* gather_row,
                    const float* obs_row, bool ssg_on, bool image) {
    const size_t N = s->N;
    cudaStream_t st = s->stream;
    const int nxx = s->d.nxx, nzz = s->d.nzz, nzh = s->nzh;
    const float norm = (float)(1.0 / ((double)nxx * nzz));
    {
        VzArgsA a{};
        a.nxx = nxx; a.nzz = nzz; a.nzh = nzh; a.L = s->Lzv; a.pl = s->pz; a.plc = s->pzc;
        a.HzM = s->cHzM; a.i_az = s->i_az; a.i_bz = s->i_bz;
        a.aux_spec = w.aux_pending ? w.aux_spec : nullptr;
        a.aux = w.aux(N); a.vz = w.vz(N); a.psi_vz = w.fivzz(N); a.Dx = w.Dx(N);
        a.div = s->div; a.G = s->spec[0];
        ProfScope ps(s, QPSTD_K_ZPASS);
        launch_vz_passA(a, st);
        w.aux_pending = false;
    }
    VxsArgs xs{};
    xs.nxx = nxx; xs.nzz = nzz; xs.nzh = nzh; xs.pl = s->px; xs.kx2 = s->kxsq; xs.kz2 = s->kzsq; xs.norm = norm;
    xs.plc = s->pxc;
    // modes 0 and 1 (stationary symbols): per-kz convolution tables when built;
    // launches on exact DFTs are timed as their own kind
    auto xspec = [&](VxsArgs& a) {
        if (s->xconv && a.mode != 2) {
            a.tab0 = s->xtab[a.mode == 0 ? 0 : 3];
            a.tab1 = s->xtab[1];
            a.tab2 = s->xtab[2];
            ProfScope ps(s, QPSTD_K_XSPEC);
            launch_vz_xspec_conv(a, st);
        } else {
            ProfScope ps(s, QPSTD_K_XSPEC_EXACT);
            launch_vz_xspec(a, st);
        }
    };
    const bool lowrank = s->lr_row > 0;
    if (lowrank) {
        // low-rank form: total <- W{div} = sum_b c_b Re F^-1[Vt_b F div] / N
        LrxArgs x{};
        x.nxx = nxx; x.nzh = nzh; x.L = s->Llr; x.row = s->lr_row; x.plc = s->pxc;
        x.in = s->spec[0]; x.out = s->lr_Q; x.tab = s->lr_tab;
        {
            ProfScope ps(s, QPSTD_K_XSPEC);
            launch_lr_xconv(x, st);
        }
        LrsArgs z{};
        z.nxx = nxx; z.nzz = nzz; z.nzh = nzh; z.L = s->Llrz; z.row = s->lr_row; z.pl = s->pz;
        z.Q = s->lr_Q; z.c = s->lr_c; z.psc = s->total;
        ProfScope ps(s, QPSTD_K_ZPASS);
        launch_lr_zsum(z, st);
    } else {
        {
            VxsArgs a = xs;
            a.mode = 0; a.L = s->Lxs3;
            a.in = s->spec[0]; a.out0 = s->spec[1]; a.out1 = s->spec[2]; a.out2 = s->spec[3];
            xspec(a);
        }
        {
            VzArgsB a{};
            a.nxx = nxx; a.nzz = nzz; a.nzh = nzh; a.L = s->Lzv; a.pl = s->pz;
            a.Y2 = s->spec[1]; a.Y3 = s->spec[2]; a.Y4 = s->spec[3];
            a.div = s->div; a.y1 = s->y1; a.y2 = s->y2; a.y3c = s->y3c; a.y4c = s->y4c;
            a.total = s->total; a.T = s->spec[0];
            ProfScope ps(s, QPSTD_K_ZPASS);
            launch_vz_passB(a, st);
        }
        {
            VxsArgs a = xs;
            a.mode = 1; a.L = s->Lxs;
            a.in = s->spec[0]; a.out0 = s->spec[1];
            xspec(a);
        }
    }
    {
        VzArgsC a{};
        a.nxx = nxx; a.nzz = nzz; a.nzh = nzh; a.L = s->Lzv; a.pml = s->d.pml; a.pl = s->pz;
        a.Dspec = lowrank ? nullptr : s->spec[1]; a.total = s->total; a.aux = w.aux(N); a.p = w.p(N);
        // low-rank form: p += rho vp^2 dt W{div} -/+ dt tau aux (the pressure term of the
        // reference's dormant addsa_b_kernel, sgpstd-qmodeling/acsglw.cu:1542-1571)
        a.e1 = lowrank ? s->c1 : s->e1; a.e2 = s->e2; a.e3 = s->e3;
        a.sgn = (s->d.kind == QPSTD_QRTM) ? 1.f : -1.f;
        a.xs = (src != 0.f) ? s->d.xsg : -1; a.zs = s->d.zsg; a.src = src;
        if (gather_row || obs_row) { a.rec_off = s->rec_off_z; a.rec = s->rec_z; }
        a.gather_row = gather_row; a.obs_row = obs_row;
        if (ssg_on) { a.ssg = s->ssg; a.ssg_c = s->ssg_c; }
        if (image) { a.img = s->img; a.img_c = s->img_c; a.ps = s->src.p(N); }
        a.P = s->spec[2]; a.HzP = s->HzP; a.h_az = s->h_az; a.h_bz = s->h_bz; a.bbz = s->bbz;
        a.vz = w.vz(N); a.psi_pz = w.fipz(N); a.dt = s->d.dt;
        ProfScope ps(s, QPSTD_K_ZPASS);
        launch_vz_passC(a, st);
    }
    {
        ProfScope ps(s, QPSTD_K_XPASS);
        launch_ac_xpass(xargs(s, w, 0, 1, last ? 0 : 1), st);
    }
    {
        VxsArgs a = xs;
        a.L = s->Lxs;
        a.in = s->spec[2]; a.out0 = w.aux_spec;
        if (s->d.kind == QPSTD_QRTM && !(s->xconv && filter_is_ka(s, eta, t_filter))) {
            // multt_kernel, sgpstd-qrtm/acsglw.cu:1895: eta scaled by 1e-6, tt = nt*dt in float
            a.mode = 2; a.eta6 = (float)((double)eta * 1e-6); a.tao = s->d.taoc; a.dt = s->d.dt;
            a.tt = (float)t_filter * s->d.dt;
        } else {
            a.mode = 1;
        }
        if (a.mode == 2 && s->xconv) a.L = s->Lxs_exact;
        xspec(a);
        w.aux_pending = true;
    }
}

// Turn a pending aux spectrum back into the real aux field.
static void vz_finish(qpstd_shot* s, Wave& w) {
    if (!w.aux_pending) return;
    VzArgsI a{};
    a.nxx = s->d.nxx; a.nzz = s->d.nzz; a.nzh = s->nzh; a.L = s->Lzv; a.pl = s->pz;
    a.spec = w.aux_spec; a.out = w.aux(s->N);
    ProfScope ps(s, QPSTD_K_ZPASS);
    launch_vz_zinv(a, s->stream);
    w.aux_pending = false;
}

static float src_amp(qpstd_shot* s, int t) {
    return (t >= 0 && t < s->d.nt) ? (float)((double)s->rik[t] * s->d.dt * 1000.0) : 0.f;
}

// One step at source-wavelet index t.  first: no pending vz update;
// gather_row: device row for the receivers (or null); ssg_on: accumulate the
// illumination (first sweep of RTM, addsa_kernel restart==0).
static void src_step(qpstd_shot* s, int t, bool first, bool last, float* gather_row, bool ssg_on) {
    Wave& w = s->src;
    if (s->d.method == QPSTD_PLAIN) {
        plain_one(s, w, src_amp(s, t), t, s->d.etas, gather_row, nullptr, ssg_on, false);
        return;
    }
    if (s->visco) {
        vz_step(s, w, src_amp(s, t), t, s->d.etas, last, gather_row, nullptr, ssg_on, false);
        return;
    }
    {
        ProfScope ps(s, QPSTD_K_ZPASS);
        launch_ac_zpass(zargs(s, w, first ? 0 : 1, 1), s->stream);
    }
    AcXArgs x = xargs(s, w, 1, 1, last ? 0 : 1);
    x.xs = s->d.xsg;
    x.zs = s->d.zsg;
    x.src = src_amp(s, t);
    if (gather_row) {
        x.rec_off = s->rec_off;
        x.rec = s->rec;
    }
    x.gather_row = gather_row;
    if (ssg_on) {
        x.ssg = s->ssg;
        x.ssg_c = s->ssg_c;
    }
    ProfScope ps(s, QPSTD_K_XPASS);
    launch_ac_xpass(x, s->stream);
}

static void src_end(qpstd_shot* s) {
    if (s->d.method == QPSTD_PLAIN) return;
    if (s->visco) {
        vz_finish(s, s->src);
        return;
    }
    ProfScope ps(s, QPSTD_K_ZPASS);
    launch_ac_zpass(zargs(s, s->src, 1, 0), s->stream);
}

// ---- autotuning of the lines per CTA -------------------------------------------
// Every pass kernel family runs L lines per CTA; L trades resident CTAs per SM
// (latency hiding across barriers) against grid size, tail and shared memory.
// At shot creation each family's admissible L (threads <= 768, shared memory
// within the kernel's limit, powers of two where the tile needs it) are timed
// in whole pipelined steps on the shot's own buffers -- zero state, no source
// (t = -1), no recording, so every field stays zero -- one family after the
// other, keeping the fastest.  Results are cached per grid shape for the
// process.  QPSTD_AUTOTUNE=0 keeps the built-in choice.
namespace {
// One tuned kernel family: its lines per CTA and, for the acoustic passes,
// whether the epilogue inputs are staged in shared memory (staging hides
// their loads behind the transforms but takes shared memory that would hold
// more resident CTAs).
struct Knob {
    int* L;
    bool pow2;
    int tx;              // threads per line
    size_t per_line;     // shared bytes per line without staging
    size_t budget;       // shared bytes the kernel may use
    bool* stage = nullptr;
    size_t stage_bytes = 0;  // extra shared bytes per line when staging
};
std::mutex g_tune_mu;
std::map<std::vector<int>, std::vector<int>> g_tune_cache;

int lmax_of(int tx, size_t per_line, size_t budget) {
    return std::max(1, std::min(QP_MAXTHREADS / std::max(tx, 1), (int)(budget / std::max<size_t>(per_line, 1))));
}
}  // namespace

static float time_steps(qpstd_shot* s, int warm, int n) {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    src_begin(s);
    for (int i = 0; i < warm; i++) src_step(s, -1, i == 0, false, nullptr, false);
    cudaEventRecord(a, s->stream);
    for (int i = 0; i < n; i++) src_step(s, -1, false, i == n - 1, nullptr, false);
    cudaEventRecord(b, s->stream);
    src_end(s);
    float ms = -1.f;
    if (cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

// The tuned kernel families of a shot.
static std::vector<Knob> shot_knobs(qpstd_shot* s) {
    const size_t stz = (size_t)40 * s->d.nzz, stx = xstage_bytes(s->visco, s->d.nxx);
    std::vector<Knob> knobs;
    const size_t vzb = 160 * 1024, acb = QP_SMEM_DYN_MAX;
    if (s->visco) {
        const int mz = std::max(s->pz.m, s->pzc.m), tz = std::max(s->pz.tx, s->pzc.tx);
        const FFTPlanDev& pxs = s->xconv ? s->pxc : s->px;
        knobs.push_back({&s->Lzv, false, tz, (size_t)16 * mz, vzb});  // z passes A-C share L
        knobs.push_back({&s->Lxs3, true, pxs.tx, (size_t)16 * pxs.m, vzb});
        knobs.push_back({&s->Lxs, true, pxs.tx, (size_t)8 * pxs.m, vzb});
        if (s->xconv && s->d.kind == QPSTD_QRTM)
            knobs.push_back({&s->Lxs_exact, true, s->px.tx, (size_t)8 * s->px.m, vzb});
    } else {
        knobs.push_back({&s->Lzp, false, s->pzc.tx, (size_t)8 * s->pzc.m, acb, &s->stage_z, stz});
    }
    knobs.push_back({&s->Lx, true, s->pxc.tx, (size_t)8 * s->pxc.m, acb, &s->stage_x, stx});
    return knobs;
}

// QPSTD_TUNE_STAGING=0 keeps epilogue staging off in every tuned pass.
static bool staging_allowed() {
    const char* env = getenv("QPSTD_TUNE_STAGING");
    return !(env && env[0] == '0');
}

// Admissible (staging, L) pairs of a knob.
static std::vector<std::pair<int, int>> knob_pairs(const Knob& k) {
    std::vector<std::pair<int, int>> out;
    const bool staging = k.stage && staging_allowed();
    for (int st = 0; st <= (staging ? 1 : 0); st++) {
        const size_t per = k.per_line + (st ? k.stage_bytes : 0);
        if (per > k.budget) continue;  // staging does not fit beside one line
        const int lmax = lmax_of(k.tx, per, k.budget);
        for (int L : {1, 2, 3, 4, 6, 8, 12, 16})
            if (L <= lmax && (!k.pow2 || (L & (L - 1)) == 0)) out.push_back({st, L});
    }
    return out;
}

static void knob_set(const Knob& k, std::pair<int, int> c) {
    if (k.stage) *k.stage = c.first != 0;
    *k.L = c.second;
}

// Zero state and scratch spectra (cudaMalloc leaves them undefined) so that
// tuning steps keep every field zero.
static void tune_prepare(qpstd_shot* s) {
    for (int k = 0; k < 4; k++)
        if (s->spec[k]) cudaMemsetAsync(s->spec[k], 0, sizeof(float2) * (size_t)s->d.nxx * s->nzh, s->stream);
    cudaMemsetAsync(s->src.st, 0, sizeof(float) * 9 * s->N, s->stream);
}

static int autotune(qpstd_shot* s) {
    const char* env = getenv("QPSTD_AUTOTUNE");
    if (s->d.method != QPSTD_FUSED || (env && env[0] == '0')) return QPSTD_OK;
    std::vector<Knob> knobs = shot_knobs(s);
    // cached per shape: L * 2 + staging
    const std::vector<int> key = {s->d.kind, s->d.nxx, s->d.nzz};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end() && it->second.size() == knobs.size()) {
            for (size_t i = 0; i < knobs.size(); i++) {
                *knobs[i].L = it->second[i] >> 1;
                if (knobs[i].stage) *knobs[i].stage = it->second[i] & 1;
            }
            return QPSTD_OK;
        }
    }
    tune_prepare(s);
    const bool prof = s->prof;
    s->prof = false;
    for (Knob& k : knobs) {
        // the current (staging, L) first, then every other admissible pair
        if (k.stage && !staging_allowed()) *k.stage = false;
        std::vector<std::pair<int, int>> cand = {{k.stage ? (int)*k.stage : 0, *k.L}};
        for (const auto& c : knob_pairs(k))
            if (c != cand[0]) cand.push_back(c);
        // Two rounds over the candidates, each candidate's best of its two
        // timings kept: a drift of the clocks during tuning then weighs on
        // every candidate alike instead of on the ones timed first.
        std::vector<float> tm(cand.size(), 1e30f);
        for (int round = 0; round < 2; round++)
            for (size_t ci = 0; ci < cand.size(); ci++) {
                knob_set(k, cand[ci]);
                const float t = time_steps(s, 1, 3);
                if (t > 0.f) tm[ci] = std::min(tm[ci], t);
            }
        std::pair<int, int> best = cand[0];
        float tbest = 1e30f;
        for (size_t ci = 0; ci < cand.size(); ci++) {
            // The shot is timed alone, but staging holds shared memory that the
            // CTAs of other shots on the GPU could use: a staged choice has to
            // win by 5 % (on the 64-shot Q-RTM batch, x-pass staging measured
            // +0 % alone and -1.3 % in the batch).
            const float t = cand[ci].first ? tm[ci] * 1.05f : tm[ci];
            if (t < tbest) {
                tbest = t;
                best = cand[ci];
            }
        }
        knob_set(k, best);
    }
    s->prof = prof;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    std::vector<int> val;
    for (Knob& k : knobs) val.push_back(*k.L * 2 + (k.stage && *k.stage ? 1 : 0));
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = val;
    return QPSTD_OK;
}

// Advance the source wavefield over steps t0 .. t0+n-1 (source wavelet index t).
// gather: device rows for each step (row t-t0), or null.
static int advance_src(qpstd_shot* s, int t0, int n, float* gather, bool ssg_on) {
    if (n <= 0) return QPSTD_OK;
    src_begin(s);
    for (int t = t0; t < t0 + n; t++)
        src_step(s, t, t == t0, t == t0 + n - 1, gather ? gather + (size_t)(t - t0) * s->d.nr : nullptr, ssg_on);
    src_end(s);
    if (s->plain_err) return fail(QPSTD_ECUDA, "plain step failed (cuFFT or launch)");
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return QPSTD_OK;
}

// Device bytes qpstd_shot_create takes for d (the buffers above, each rounded
// to 256 bytes, plus 1 MiB for the small tables); the plain form adds its
// complex scratch and a cuFFT work area of the same order.
extern "C" long long qpstd_shot_bytes(const qpstd_shot_desc* d) {
    if (!d || d->nxx < 1 || d->nzz < 1 || d->nt < 1) return -1;
    const bool visco = d->kind == QPSTD_VAPS || d->kind == QPSTD_QRTM;
    const bool rtm = d->kind == QPSTD_ARTM || d->kind == QPSTD_QRTM;
    const double N = (double)d->nxx * d->nzz, nzh = d->nzz / 2 + 1, NS = d->nxx * nzh;
    const double nr = std::max(d->nr, 1), nx = d->nxx - 2 * d->pml, nz = d->nzz - 2 * d->pml;
    const bool fused = d->method != QPSTD_PLAIN;
    HostPlan cx, cz, ex, ez;
    if (fused && (build_conv_plan_host(d->nxx, cx, true) || build_conv_plan_host(d->nzz, cz) ||
                  build_plan_host(d->nxx, ex, true) || build_plan_host(d->nzz, ez)))
        return -1;  // no fused plan for these lengths
    double f = (rtm ? 18.0 : 9.0) * N + 6.0 * N;                       // wavefields; div, Lz, bbx, bbz, c1, c2
    if (fused) {
        f += 2.0 * (cx.m + cz.m) + 6.0 * (cx.m + cz.m);                // convolution plans and multipliers
        f += 2.0 * (2.0 * ex.m + d->nxx) + 2.0 * (2.0 * ez.m + d->nzz);  // exact plans (twiddles, chirp, bhat)
    }
    f += 16.0 * (d->nxx + d->nzz);                                     // CPML profiles, squared wavenumbers
    if (visco) {
        f += 8.0 * N + 2.0 * NS * (rtm ? 6 : 5) + 4.0 * (d->nxx + d->nzz);
        if (fused && ex.blue) f += 4.0 * nzh * (cx.m / 2 + 1);         // per-kz convolution tables
    }
    f += (double)d->nt * nr;                                           // gather
    if (rtm) f += (double)d->snaps * 8.0 * N + (double)d->nt * nr + 4.0 * nx * nz;
    if (d->method == QPSTD_PLAIN) f += 20.0 * N;
    return (long long)(4.0 * f) + 32 * 256 + (1ll << 20);
}

// Modeling in slices, for callers that interleave many shots: steps t0 .. t0+n-1
// of the source wavefield with the gather rows recorded on the device (row t of
// s->gather).  The slice at t0 = 0 starts the pipeline and the slice that
// reaches nt completes it, so consecutive slices equal one advance over 0..nt-1.
int model_slice(qpstd_shot* s, int t0, int n) {
    if (!s || n <= 0 || t0 < 0 || t0 + n > s->d.nt) return fail(QPSTD_EINVAL, "bad modeling slice");
    const int nt = s->d.nt, nr = s->d.nr;
    if (t0 == 0) {
        s->launches = 0;
        src_begin(s);
    }
    for (int t = t0; t < t0 + n; t++)
        src_step(s, t, t == 0, t == nt - 1, nr > 0 ? s->gather + (size_t)t * nr : nullptr, false);
    if (t0 + n == nt) src_end(s);
    if (s->plain_err) return fail(QPSTD_ECUDA, "plain step failed (cuFFT or launch)");
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return QPSTD_OK;
}

extern "C" int qpstd_shot_pipeline_begin(qpstd_shot* s) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    s->launches = 0;
    s->pipe_first = true;
    src_begin(s);
    return QPSTD_OK;
}

extern "C" int qpstd_shot_pipeline_step(qpstd_shot* s, int t, int last) {
    if (!s || t < 0) return fail(QPSTD_EINVAL, "bad pipeline step");
    src_step(s, t, s->pipe_first, last != 0, nullptr, false);
    s->pipe_first = false;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return QPSTD_OK;
}

extern "C" int qpstd_shot_pipeline_end(qpstd_shot* s) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    src_end(s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return QPSTD_OK;
}

// One receiver-side step (firsturn / youturn): injected at the receivers from
// obs row `row`, then imaged against the source wavefield.  The receiver
// wavefield stays pipelined between calls (its vz update is folded into the
// next call's z pass); nothing else reads it.
static int receiver_step(qpstd_shot* s, int row, bool first) {
    Wave& w = s->rcv;
    cudaStream_t st = s->stream;
    if (s->d.method == QPSTD_PLAIN) {
        plain_one(s, w, 0.f, row, s->d.etar, nullptr, s->obs + (size_t)row * s->d.nr, false, true);
        if (s->plain_err) return fail(QPSTD_ECUDA, "plain step failed (cuFFT or launch)");
        return QPSTD_OK;
    }
    if (s->visco) {
        // addsa_b_kernel + multt_kernel(etar, nt = row), sgpstd-qrtm/acsglw.cu:745-776, 907-940
        vz_step(s, w, 0.f, row, s->d.etar, false, nullptr, s->obs + (size_t)row * s->d.nr, false, true);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        return QPSTD_OK;
    }
    {
        ProfScope ps(s, QPSTD_K_ZPASS);
        launch_ac_zpass(zargs(s, w, first ? 0 : 1, 1), st);
    }
    AcXArgs x = xargs(s, w, 1, 1, 1);
    x.rec_off = s->rec_off;
    x.rec = s->rec;
    x.obs_row = s->obs + (size_t)row * s->d.nr;
    x.img = s->img;
    x.img_c = s->img_c;
    x.ps = s->src.p(s->N);
    {
        ProfScope ps(s, QPSTD_K_XPASS);
        launch_ac_xpass(x, st);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return QPSTD_OK;
}

extern "C" int qpstd_shot_advance_device(qpstd_shot* s, int t0, int nsteps) {
    if (!s || nsteps < 0 || nsteps > s->d.nt || t0 < 0) return fail(QPSTD_EINVAL, "bad advance arguments");
    s->launches = 0;
    return advance_src(s, t0, nsteps, s->d.nr > 0 ? s->gather : nullptr, false);
}

extern "C" int qpstd_shot_advance(qpstd_shot* s, int t0, int nsteps, float* gather) {
    int rc = qpstd_shot_advance_device(s, t0, nsteps);
    if (rc) return rc;
    if (gather && s->d.nr > 0)
        CK(cudaMemcpyAsync(gather, s->gather, sizeof(float) * (size_t)nsteps * s->d.nr, cudaMemcpyDeviceToHost,
                           s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return QPSTD_OK;
}

extern "C" long long qpstd_shot_launch_count(const qpstd_shot* s) { return s ? s->launches : -1; }

// Low-rank form of the pressure term (see qpstd.h).  c_b(x) = sum_a U[x][a] A[a][b]
// is formed once in FP64 (the reference accumulates these sums in double,
// sumlw_kernel / sumlw2_kernel, sgpstd-qmodeling/acsglw.cu:1444-1497); each V_b,
// mirrored to the full kx range (consist_Vt, sglowrank.c:103-145), becomes a
// per-kz convolution table on the x convolution plan.
extern "C" int qpstd_shot_set_lowrank(qpstd_shot* s, int row, int col, const float* U, const float* V,
                                      const double* A) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    if (!s->visco || s->d.method != QPSTD_FUSED)
        return fail(QPSTD_EINVAL, "the low-rank form applies to fused constant-Q shots (VAPS, QRTM)");
    if (row < 1 || col < 1 || row > 16 || col > 16 || !U || !V || !A)
        return fail(QPSTD_EINVAL, "low-rank factors: 1 <= row, col <= 16 and U, V, A non-null");
    if (s->lr_row) return fail(QPSTD_EINVAL, "the shot already runs the low-rank form");
    const int nxx = s->d.nxx, nzz = s->d.nzz, nzh = s->nzh, nxh = nxx / 2 + 1;
    const size_t N = s->N;
    const int mc = s->pxc.m, mh = mc / 2 + 1;
    int rc = QPSTD_OK;
    float* c = dalloc(s, (size_t)row * N, &rc);
    float* tab = c ? dalloc(s, (size_t)row * nzh * mh, &rc) : nullptr;
    float* Q = tab ? dalloc(s, (size_t)row * 2 * nxx * nzh, &rc) : nullptr;
    float* Vd = Q ? dalloc(s, (size_t)row * nxh * nzh, &rc) : nullptr;
    if (!Vd) return rc;
    std::vector<float> hc((size_t)row * N);
    for (size_t x = 0; x < N; x++)
        for (int b = 0; b < row; b++) {
            double acc = 0.0;
            for (int a = 0; a < col; a++) acc += (double)U[x * col + a] * A[(size_t)a * row + b];
            hc[(size_t)b * N + x] = (float)acc;
        }
    CK(cudaMemcpy(c, hc.data(), sizeof(float) * hc.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(Vd, V, sizeof(float) * (size_t)row * nxh * nzh, cudaMemcpyHostToDevice));
    VtabArgs a{};
    a.nxx = nxx; a.nzz = nzz; a.nzh = nzh;
    a.pl = s->px; a.plc = s->pxc; a.kx2 = s->kxsq; a.kz2 = s->kzsq;
    a.norm = (float)(1.0 / ((double)nxx * nzz));
    a.L = choose_L(nzh, std::max(s->px.m, mc), std::max(s->px.tx, s->pxc.tx), 1, false);
    a.sym = 4;
    a.nxh = nxh;
    for (int b = 0; b < row; b++) {
        a.V = Vd + (size_t)b * nxh * nzh;
        a.out = tab + (size_t)b * nzh * mh;
        launch_vz_convtab(a, s->stream);
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "low-rank tables");
    s->lr_c = c;
    s->lr_tab = tab;
    s->lr_Q = reinterpret_cast<float2*>(Q);
    s->Llr = choose_L(nzh, mc, s->pxc.tx, 2, true);
    s->Llrz = choose_L((nxx + 1) / 2, s->pz.m, s->pz.tx, 2, false);
    s->lr_row = row;
    return QPSTD_OK;
}

extern "C" long long qpstd_shot_info(const qpstd_shot* s, int key) {
    if (!s) return -1;
    switch (key) {
        case QPSTD_INFO_X_CONV_M: return s->pxc.m;
        case QPSTD_INFO_X_CONV_MAXRADIX: return plan_max_radix(s->pxc);
        case QPSTD_INFO_X_EXACT_M: return s->px.m;
        case QPSTD_INFO_X_EXACT_BLUE: return s->px.blue;
        case QPSTD_INFO_X_SPEC_CONV: return s->xconv ? 1 : 0;
        case QPSTD_INFO_Z_EXACT_M: return s->pz.m;
        case QPSTD_INFO_Z_EXACT_MAXRADIX: return plan_max_radix(s->pz);
        case QPSTD_INFO_Z_CONV_M: return s->pzc.m;
        default: return -1;
    }
}

extern "C" void* qpstd_shot_stream(qpstd_shot* s) { return s ? (void*)s->stream : nullptr; }

extern "C" int qpstd_shot_set_profiling(qpstd_shot* s, int on) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    s->prof = on != 0;
    return QPSTD_OK;
}

extern "C" int qpstd_shot_profile_read(qpstd_shot* s, int nkinds, double* ms, long long* count) {
    if (!s || nkinds < 1 || !ms || !count) return fail(QPSTD_EINVAL, "bad profile arguments");
    CK(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < nkinds; k++) {
        ms[k] = 0.0;
        count[k] = 0;
    }
    for (auto& t : s->timed) {
        float v = 0.f;
        cudaEventElapsedTime(&v, t.a, t.b);
        if (t.kind >= 0 && t.kind < nkinds) {
            ms[t.kind] += v;
            count[t.kind] += 1;
        }
        s->evpool.push_back(t.a);
        s->evpool.push_back(t.b);
    }
    s->timed.clear();
    return QPSTD_OK;
}
extern "C" long long qpstd_shot_forward_steps(const qpstd_shot* s) { return s ? s->fwd_steps : -1; }
int shot_set_priority(qpstd_shot* s, int prio) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    CK(cudaStreamSynchronize(s->stream));
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio));
    if (s->plain.have_plan && cufftSetStream(s->plain.plan, st) != CUFFT_SUCCESS) {
        cudaStreamDestroy(st);
        return fail(QPSTD_ECUDA, "cufftSetStream failed");
    }
    cudaStreamDestroy(s->stream);
    s->stream = st;
    return QPSTD_OK;
}

extern "C" int qpstd_shot_sync(qpstd_shot* s) {
    if (!s) return fail(QPSTD_EINVAL, "null shot");
    CK(cudaStreamSynchronize(s->stream));
    return QPSTD_OK;
}

extern "C" int qpstd_shot_set_obs(qpstd_shot* s, const float* obs) {
    if (!s || !obs || !s->rtm) return fail(QPSTD_EINVAL, "set_obs needs an RTM shot and data");
    if (s->d.nr > 0)
        CK(cudaMemcpyAsync(s->obs, obs, sizeof(float) * (size_t)s->d.nt * s->d.nr, cudaMemcpyHostToDevice,
                           s->stream));
    return QPSTD_OK;
}

// Revolve-driven RTM, the action loop of sgpstd-qrtm/acps4.cu:449-905 and
// sgpstd-qrtm/acsglw.cu:470-1039, as a resumable state machine: rtm_begin()
// resets the shot, each rtm_action() enqueues one revolve action on the
// shot's stream and returns 1 once revolve terminates.  A batch interleaves
// the actions of its shots, so their work overlaps on the device.
int rtm_begin(qpstd_shot* s) {
    if (!s || !s->rtm) return fail(QPSTD_EINVAL, "not an RTM shot");
    const size_t N = s->N, NI = (size_t)s->nx * s->nz;
    cudaStream_t st = s->stream;
    s->launches = 0;
    s->fwd_steps = 0;
    CK(cudaMemsetAsync(s->src.st, 0, sizeof(float) * 9 * N, st));
    CK(cudaMemsetAsync(s->rcv.st, 0, sizeof(float) * 9 * N, st));
    CK(cudaMemsetAsync(s->img, 0, sizeof(float) * 4 * NI, st));
    s->src.aux_pending = s->rcv.aux_pending = false;
    s->run = RtmRun();
    s->run.rv = Revolve(s->d.nt, s->d.snaps);
    return QPSTD_OK;
}

int rtm_action(qpstd_shot* s) {
    RtmRun& r = s->run;
    if (r.done) return 1;
    const size_t N = s->N;
    cudaStream_t st = s->stream;
    int rc;
    if (r.adv_left > 0) {
        // continue an advance in slices so that the shots of a batch interleave
        const int n = std::min(r.adv_left, r.slice);
        for (int i = 0; i < n; i++) {
            const int t = r.adv_t++;
            src_step(s, t, t == r.adv_t0, r.adv_left == 1, nullptr, r.first_sweep);
            r.adv_left--;
        }
        if (r.adv_left == 0) src_end(s);
        if (s->plain_err) return fail(QPSTD_ECUDA, "plain step failed (cuFFT or launch)");
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        return 0;
    }
    const RevolveAction act = r.rv.next();
    if (act == RV_TAKESHOT) {
        float* slot = s->store + (size_t)r.rv.check() * 8 * N;
        CK(cudaMemcpyAsync(slot, s->src.st, sizeof(float) * 8 * N, cudaMemcpyDeviceToDevice, st));
        if (r.rv.capo() == 0) {
            // checkpoint 0 also holds the first source sample (acsglw.cu:493-500)
            ProfScope ps(s, QPSTD_K_OTHER);
            add_point_kernel<<<1, 1, 0, st>>>(slot + (size_t)s->d.xsg * s->d.nzz + s->d.zsg,
                                              (float)((double)s->rik[0] * 1000.0 * s->d.dt));
        }
    } else if (act == RV_ADVANCE) {
        const int n = r.rv.capo() - r.ts + 1;
        s->fwd_steps += n;
        if (r.slice >= n) {
            if ((rc = advance_src(s, r.ts, n, nullptr, r.first_sweep))) return rc;
        } else if (n > 0) {
            src_begin(s);
            r.adv_t0 = r.adv_t = r.ts;
            r.adv_left = n;
        }
        r.ts = r.rv.capo() + 1;
    } else if (act == RV_FIRSTURN || act == RV_YOUTURN) {
        if (act == RV_FIRSTURN) r.first_sweep = false;
        const int row = (act == RV_FIRSTURN) ? s->d.nt - 1 : r.rv.capo();
        if ((rc = receiver_step(s, row, r.first_rcv))) return rc;
        r.first_rcv = false;
    } else if (act == RV_RESTORE) {
        const float* slot = s->store + (size_t)r.rv.check() * 8 * N;
        CK(cudaMemcpyAsync(s->src.st, slot, sizeof(float) * 8 * N, cudaMemcpyDeviceToDevice, st));
        s->src.aux_pending = false;
        r.ts = r.rv.capo() + 1;
    } else if (act == RV_TERMINATE) {
        r.done = true;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        return 1;
    } else {
        char buf[96];
        snprintf(buf, sizeof(buf), "irregular termination of revolve (info %d)", r.rv.info());
        return fail(QPSTD_EREVOLVE, buf);
    }
    return 0;
}

extern "C" int qpstd_shot_rtm_device(qpstd_shot* s) {
    int rc = rtm_begin(s);
    if (rc) return rc;
    while ((rc = rtm_action(s)) == 0) {
    }
    return rc < 0 ? rc : QPSTD_OK;
}

extern "C" int qpstd_shot_get_image(qpstd_shot* s, float* img, float* ssg) {
    if (!s || !s->rtm) return fail(QPSTD_EINVAL, "not an RTM shot");
    const size_t NI = (size_t)s->nx * s->nz;
    if (img) CK(cudaMemcpyAsync(img, s->img, sizeof(float) * NI, cudaMemcpyDeviceToHost, s->stream));
    if (ssg) CK(cudaMemcpyAsync(ssg, s->ssg, sizeof(float) * NI, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return QPSTD_OK;
}

// ---------------------------------------------------------------------------
extern "C" int qpstd_model_shot(const qpstd_shot_desc* d, float* gather, float* state) {
    if (!d) return fail(QPSTD_EINVAL, "null descriptor");
    if (d->kind != QPSTD_APS && d->kind != QPSTD_VAPS) return fail(QPSTD_EINVAL, "modeling needs APS or VAPS");
    qpstd_shot* s = nullptr;
    int rc = qpstd_shot_create(d, &s);
    if (rc) return rc;
    rc = qpstd_shot_advance(s, 0, d->nt, gather);
    if (!rc && state) rc = qpstd_shot_get_state(s, state);
    qpstd_shot_destroy(s);
    return rc;
}

extern "C" int qpstd_rtm_shot(const qpstd_shot_desc* d, const float* obs, float* img, float* ssg) {
    if (!d || !obs) return fail(QPSTD_EINVAL, "null argument");
    if (d->kind != QPSTD_ARTM && d->kind != QPSTD_QRTM) return fail(QPSTD_EINVAL, "RTM needs ARTM or QRTM");
    qpstd_shot* s = nullptr;
    int rc = qpstd_shot_create(d, &s);
    if (rc) return rc;
    if (!(rc = qpstd_shot_set_obs(s, obs)))
        if (!(rc = qpstd_shot_rtm_device(s))) rc = qpstd_shot_get_image(s, img, ssg);
    qpstd_shot_destroy(s);
    return rc;
}

// ---------------------------------------------------------------------------
// 5-point Laplacian filter (filter_image, sgpstd-qrtm/acsglw.cu:1872-1893),
// bounds-checked so no write leaves the nx*nz image.
__global__ void filter_image_kernel(int nx, int nz, float rdx2, float rdz2, const float* __restrict__ img,
                                    float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * nz) return;
    const int ix = i / nz, iz = i - ix * nz;
    if (ix == 0 || iz == 0 || ix == nx - 1 || iz == nz - 1) {
        out[i] = 0.f;
        return;
    }
    out[i] = (img[i + 1] + img[i - 1] - 2.f * img[i]) * rdz2 + (img[i + nz] + img[i - nz] - 2.f * img[i]) * rdx2;
}

extern "C" int qpstd_pml_profiles(int pml, float fd, int nxx, int nzz, float dx, float dz, float dt, float* out) {
    if (pml < 2 || nxx < 2 * pml + 1 || nzz < 2 * pml + 1 || !out) return fail(QPSTD_EINVAL, "bad CPML grid");
    std::vector<double> v[8];  // i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz
    pml_coeffs(pml, fd, nxx, nzz, dx, dz, dt, v);
    const int order[8] = {0, 1, 4, 5, 2, 3, 6, 7};  // x tables, then z tables
    size_t q = 0;
    for (int k : order)
        for (double x : v[k]) out[q++] = (float)x;
    return QPSTD_OK;
}

extern "C" int qpstd_filter_image(int nx, int nz, float dx, float dz, const float* img, float* imgf) {
    if (nx < 1 || nz < 1 || !img || !imgf) return fail(QPSTD_EINVAL, "bad filter arguments");
    const size_t n = (size_t)nx * nz;
    float *a = nullptr, *b = nullptr;
    CK(cudaMalloc(&a, 8 * n));
    b = a + n;
    cudaError_t e = cudaMemcpy(a, img, 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        filter_image_kernel<<<(unsigned)((n + 255) / 256), 256>>>(nx, nz, 1.f / (dx * dx), 1.f / (dz * dz), a, b);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(imgf, b, 4 * n, cudaMemcpyDeviceToHost);
    cudaFree(a);
    if (e != cudaSuccess) return cuda_fail(e, "filter_image");
    return QPSTD_OK;
}

// Source-normalised imaging condition r / (s + sigma^2): the reference
// accumulates the cross-correlation r (img_sp) and the source illumination s
// (ssg_sp) and leaves the division to the user; the stabilisation sigma^2 keeps
// unilluminated points finite.
__global__ void normalize_image_kernel(size_t n, float sigma2, const float* __restrict__ img,
                                       const float* __restrict__ ssg, float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = img[i] / (ssg[i] + sigma2);
}

extern "C" int qpstd_normalize_image(int nx, int nz, float sigma2, const float* img, const float* ssg, float* out) {
    if (nx < 1 || nz < 1 || !img || !ssg || !out) return fail(QPSTD_EINVAL, "bad normalisation arguments");
    const size_t n = (size_t)nx * nz;
    float* a = nullptr;
    CK(cudaMalloc(&a, 12 * n));
    cudaError_t e = cudaMemcpy(a, img, 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(a + n, ssg, 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        normalize_image_kernel<<<(unsigned)((n + 255) / 256), 256>>>(n, sigma2, a, a + n, a + 2 * n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, a + 2 * n, 4 * n, cudaMemcpyDeviceToHost);
    cudaFree(a);
    if (e != cudaSuccess) return cuda_fail(e, "normalize_image");
    return QPSTD_OK;
}
