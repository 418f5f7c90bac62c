// plain.cu -- the plain form of the step: cuFFT 2-D C2C transforms and
// elementwise kernels in the reference's order.
//
// This is the per-shot baseline the fused passes are measured against.  It
// follows sgpstd-qmodeling/acps4.cu:517-607 (acoustic) and
// sgpstd-qmodeling/acsglw.cu:517-645 / sgpstd-qrtm/acsglw.cu:511-657
// (constant-Q) transform for transform: 9 2-D C2C FFTs per acoustic step, 14
// per constant-Q step, with the complex intermediates kept complex exactly
// where the reference keeps them (sumpxpz adds both parts).  The elementwise
// kernels are one thread per grid point in x-major order (coalesced), unlike
// the reference's ix-fastest 16x16 blocks.
#include <cufft.h>

#include "pass_common.cuh"
#include "plain.h"
#include "shot.h"

namespace qp {

namespace {

constexpr int TB = 256;

__device__ __forceinline__ float2 pmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void k_fuzhi2(int N, const float* __restrict__ a, const float* __restrict__ b, float2* da, float2* db) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    da[i] = make_float2(a[i], 0.f);
    if (db) db[i] = make_float2(b[i], 0.f);
}

// shift_vxz_kernel / shift_pxz_kernel: out = H(k) in / N (acps4.cu:1047, 1210)
__global__ void k_shift(int nxx, int nzz, float invN, const float2* __restrict__ in_x, const float2* __restrict__ in_z,
                        const float2* __restrict__ Hx, const float2* __restrict__ Hz, float2* out_x, float2* out_z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxx * nzz) return;
    const int ix = i / nzz, iz = i - ix * nzz;
    const float2 a = pmul(in_x[i], Hx[ix]);
    const float2 b = pmul(in_z[i], Hz[iz]);
    out_x[i] = make_float2(a.x * invN, a.y * invN);
    out_z[i] = make_float2(b.x * invN, b.y * invN);
}

// update_vxx_vzz + sumpxpz (acps4.cu:1111, 1146)
__global__ void k_updv(int nxx, int nzz, float* fivxx, float* fivzz, const float* __restrict__ iax,
                       const float* __restrict__ ibx, const float* __restrict__ iaz, const float* __restrict__ ibz,
                       float2* dx, float2* dz, float2* div) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxx * nzz) return;
    const int ix = i / nzz, iz = i - ix * nzz;
    float2 a = dx[i], b = dz[i];
    const float fx = ibx[ix] * fivxx[i] + iax[ix] * a.x;
    const float fz = ibz[iz] * fivzz[i] + iaz[iz] * b.x;
    fivxx[i] = fx;
    fivzz[i] = fz;
    a.x += fx;
    b.x += fz;
    div[i] = make_float2(a.x + b.x, a.y + b.y);
}

// isotropic symbols: 0 k^2, 1 (k^2)^(1/32), 2 (k^2)^(33/32), 3 (k^2)^0.505,
// 4 stabilised filter (multt_kernel, sgpstd-qrtm/acsglw.cu:1895)
__device__ __forceinline__ float iso_symbol(int kind, float k2, float eta6, float tao, float dt, float tt) {
    if (kind == 0) return k2;
    const float lk = log2f(k2);
    if (kind == 1) return exp2f(lk * (1.f / 32.f));
    if (kind == 2) return k2 * exp2f(lk * (1.f / 32.f));
    const float ka = exp2f(0.505f * lk);
    if (kind == 3) return ka;
    return ka - 2.f * eta6 * ka * (1.f + tao * dt * ka) / (expf(-tao * tt * ka) + eta6 * expf(tao * dt * ka));
}

// multtt_kernel (acps4.cu:1709): out_j = in * sym_j / N for up to three symbols
__global__ void k_mult(int nxx, int nzz, float invN, const float* __restrict__ kx2, const float* __restrict__ kz2,
                       const float2* __restrict__ in, int s0, float2* o0, int s1, float2* o1, int s2, float2* o2,
                       float eta6, float tao, float dt, float tt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxx * nzz) return;
    const int ix = i / nzz, iz = i - ix * nzz;
    const float k2 = kx2[ix] + kz2[iz];
    const float2 v = in[i];
    float f = iso_symbol(s0, k2, eta6, tao, dt, tt) * invN;
    o0[i] = make_float2(v.x * f, v.y * f);
    if (o1) {
        f = iso_symbol(s1, k2, eta6, tao, dt, tt) * invN;
        o1[i] = make_float2(v.x * f, v.y * f);
    }
    if (o2) {
        f = iso_symbol(s2, k2, eta6, tao, dt, tt) * invN;
        o2[i] = make_float2(v.x * f, v.y * f);
    }
}

// sum_total (acsglw.cu:1213) with the coefficient fields of the shot
__global__ void k_sum_total(int N, const float2* __restrict__ div, const float2* __restrict__ y2,
                            const float2* __restrict__ y3, const float2* __restrict__ y4, const float* __restrict__ c1,
                            const float* __restrict__ c2, const float* __restrict__ c3, const float* __restrict__ c4,
                            float* total, float2* total_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float t = c1[i] * div[i].x + c2[i] * y2[i].x - (c3[i] * y3[i].x + c4[i] * y4[i].x);
    total[i] = t;
    total_c[i] = make_float2(t, 0.f);
}

// addsa_kernel / addsa_b_kernel pressure update (acps4.cu:1462, acsglw.cu:1500,
// qrtm acsglw.cu:1769); illumination on the interior when ssg != null.
__global__ void k_padd(int nxx, int nzz, int pml, int visco, float sgn, float* p, const float2* __restrict__ div,
                       const float2* __restrict__ lap, const float* __restrict__ c1, const float* __restrict__ c2,
                       const float* __restrict__ total, const float* __restrict__ e1, const float* __restrict__ e2,
                       const float* __restrict__ e3, const float* __restrict__ aux, int xs, int zs, float src,
                       float* ssg, float* ssg_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxx * nzz) return;
    const int ix = i / nzz, iz = i - ix * nzz;
    float pn;
    if (!visco)
        pn = p[i] + c1[i] * (div[i].x - c2[i] * lap[i].x);
    else
        pn = p[i] + e1[i] * (total[i] + sgn * e2[i] * lap[i].x) + sgn * e3[i] * aux[i];
    if (ix == xs && iz == zs) pn += src;
    p[i] = pn;
    const int nz = nzz - 2 * pml;
    if (ssg && ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml)
        kahan_add(ssg, ssg_c, (size_t)(ix - pml) * nz + (iz - pml), pn * pn);
}

// receivers: record p, or overwrite it with observed data (winning index per cell)
__global__ void k_receivers(int n, const RecEntry* __restrict__ rec, int nzz, float* p, float* gather_row,
                            const float* __restrict__ obs_row) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const RecEntry e = rec[q];
    const size_t i = (size_t)e.gx * nzz + e.gz;
    if (gather_row) gather_row[e.ir] = p[i];
    if (obs_row && e.inject) p[i] = obs_row[e.ir];
}

// vx_cal_kernel / vz_cal_kernel (acps4.cu:1274, 1305) + aux refresh + imaging
__global__ void k_vcal(int nxx, int nzz, int pml, float dt, const float* __restrict__ hax, const float* __restrict__ hbx,
                       const float* __restrict__ haz, const float* __restrict__ hbz, const float* __restrict__ bbx,
                       const float* __restrict__ bbz, const float2* __restrict__ px, const float2* __restrict__ pz,
                       float* fipx, float* fipz, float* vx, float* vz, const float2* __restrict__ auxc, float* aux,
                       const float* __restrict__ p, const float* __restrict__ ps, float* img, float* img_c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nxx * nzz) return;
    const int ix = i / nzz, iz = i - ix * nzz;
    const float sx = px[i].x, sz = pz[i].x;
    const float fx = hbx[ix] * fipx[i] + hax[ix] * sx;
    const float fz = hbz[iz] * fipz[i] + haz[iz] * sz;
    fipx[i] = fx;
    fipz[i] = fz;
    vx[i] = vx[i] + dt * bbx[i] * (sx + fx);
    vz[i] = vz[i] + dt * bbz[i] * (sz + fz);
    if (aux) aux[i] = auxc[i].x;
    const int nz = nzz - 2 * pml;
    if (img && ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml)
        kahan_add(img, img_c, (size_t)(ix - pml) * nz + (iz - pml), ps[i] * p[i]);
}

inline unsigned nblk(size_t n) { return (unsigned)((n + TB - 1) / TB); }

}  // namespace

// The 2-D C2C plan of the window (cufftPlan2d in the reference,
// sgpstd-qmodeling/acps4.cu:871-872) with its work area and the five complex
// scratch fields taken from the shot's own buffers (so a server's arena holds
// them too).
int plain_setup(qpstd_shot* s, std::string& err) {
    PlainState& P = s->plain;
    const size_t N = s->N;
    size_t ws = 0;
    if (cufftCreate(&P.plan) != CUFFT_SUCCESS) {
        err = "cufftCreate failed";
        return -1;
    }
    P.have_plan = true;
    if (cufftSetAutoAllocation(P.plan, 0) != CUFFT_SUCCESS ||
        cufftMakePlan2d(P.plan, s->d.nxx, s->d.nzz, CUFFT_C2C, &ws) != CUFFT_SUCCESS) {
        err = "cufftMakePlan2d failed";
        return -1;
    }
    void* work = nullptr;
    if (ws > 0 && shot_malloc(s, &work, ws) != cudaSuccess) {
        err = "no device memory for the cuFFT work area";
        return -1;
    }
    if ((ws > 0 && cufftSetWorkArea(P.plan, work) != CUFFT_SUCCESS) ||
        cufftSetStream(P.plan, s->stream) != CUFFT_SUCCESS) {
        err = "cufftSetWorkArea / cufftSetStream failed";
        return -1;
    }
    if (shot_malloc(s, (void**)&P.dis, sizeof(float2) * 5 * N) != cudaSuccess) {
        err = "no device memory for the plain scratch";
        return -1;
    }
    return 0;
}

// The plan only: the buffers are the shot's and go with them.
void plain_release(qpstd_shot* s) {
    PlainState& P = s->plain;
    if (P.have_plan) cufftDestroy(P.plan);
    P.have_plan = false;
    P.dis = nullptr;
}

// One full reference-order step of wavefield w.
int plain_step(qpstd_shot* s, Wave& w, float src, int t_filter, float eta, float* gather_row, const float* obs_row,
               bool ssg_on, bool image, long long* launches) {
    PlainState& P = s->plain;
    const int nxx = s->d.nxx, nzz = s->d.nzz, pml = s->d.pml;
    const size_t N = s->N;
    const float invN = (float)(1.0 / (double)N);
    cudaStream_t st = s->stream;
    float2 *d0 = P.dis, *d1 = P.dis + N, *d2 = P.dis + 2 * N, *d3 = P.dis + 3 * N, *d4 = P.dis + 4 * N;
    cufftComplex *c0 = (cufftComplex*)d0, *c1 = (cufftComplex*)d1, *c2 = (cufftComplex*)d2,
                 *c3 = (cufftComplex*)d3, *c4 = (cufftComplex*)d4;
    const bool visco = s->visco;
    long long nk = 0;
    int bad = 0;
    auto fft = [&](cufftComplex* a, cufftComplex* b, int dir) {
        bad |= cufftExecC2C(P.plan, a, b, dir) != CUFFT_SUCCESS;
        nk++;
    };
    // velocity divergence
    k_fuzhi2<<<nblk(N), TB, 0, st>>>((int)N, w.vx(N), w.vz(N), d0, d1);
    fft(c0, c0, CUFFT_FORWARD);
    fft(c1, c1, CUFFT_FORWARD);
    k_shift<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, d0, d1, P.HxM, P.HzM, d2, d3);
    fft(c2, c2, CUFFT_INVERSE);
    fft(c3, c3, CUFFT_INVERSE);
    k_updv<<<nblk(N), TB, 0, st>>>(nxx, nzz, w.fivxx(N), w.fivzz(N), s->i_ax, s->i_bx, s->i_az, s->i_bz, d2, d3, d0);
    nk += 3;
    // pressure update
    fft(c0, c1, CUFFT_FORWARD);
    float2* lap;
    if (!visco) {
        k_mult<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, s->kxsq, s->kzsq, d1, 0, d2, 0, nullptr, 0, nullptr, 0, 0, 0, 0);
        fft(c2, c2, CUFFT_INVERSE);
        lap = d2;
        nk += 1;
    } else {
        k_mult<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, s->kxsq, s->kzsq, d1, 1, d2, 0, d3, 2, d4, 0, 0, 0, 0);
        fft(c2, c2, CUFFT_INVERSE);
        fft(c3, c3, CUFFT_INVERSE);
        fft(c4, c4, CUFFT_INVERSE);
        k_sum_total<<<nblk(N), TB, 0, st>>>((int)N, d0, d2, d3, d4, s->y1, s->y2, s->y3c, s->y4c, s->total, d1);
        fft(c1, c1, CUFFT_FORWARD);
        k_mult<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, s->kxsq, s->kzsq, d1, 3, d0, 0, nullptr, 0, nullptr, 0, 0, 0,
                                         0);
        fft(c0, c0, CUFFT_INVERSE);
        lap = d0;
        nk += 2;
    }
    const float sgn = (s->d.kind == QPSTD_QRTM) ? 1.f : -1.f;
    k_padd<<<nblk(N), TB, 0, st>>>(nxx, nzz, pml, visco ? 1 : 0, sgn, w.p(N), d0, lap, s->c1, s->c2, s->total, s->e1,
                                   s->e2, s->e3, w.aux(N), (src != 0.f) ? s->d.xsg : -1, s->d.zsg, src,
                                   ssg_on ? s->ssg : nullptr, s->ssg_c);
    nk++;
    if ((gather_row || obs_row) && s->d.nr > 0) {
        k_receivers<<<nblk(s->d.nr), TB, 0, st>>>(s->d.nr, s->rec, nzz, w.p(N), gather_row, obs_row);
        nk++;
    }
    // pressure gradient, velocity update, aux
    k_fuzhi2<<<nblk(N), TB, 0, st>>>((int)N, w.p(N), nullptr, d0, nullptr);
    fft(c0, c0, CUFFT_FORWARD);
    k_shift<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, d0, d0, P.HxP, P.HzP, d1, d2);
    fft(c1, c1, CUFFT_INVERSE);
    fft(c2, c2, CUFFT_INVERSE);
    nk += 2;
    if (visco) {
        const bool q = s->d.kind == QPSTD_QRTM;
        k_mult<<<nblk(N), TB, 0, st>>>(nxx, nzz, invN, s->kxsq, s->kzsq, d0, q ? 4 : 3, d3, 0, nullptr, 0, nullptr,
                                         (float)((double)eta * 1e-6), s->d.taoc, s->d.dt, (float)t_filter * s->d.dt);
        fft(c3, c3, CUFFT_INVERSE);
        nk++;
    }
    k_vcal<<<nblk(N), TB, 0, st>>>(nxx, nzz, pml, s->d.dt, s->h_ax, s->h_bx, s->h_az, s->h_bz, s->bbx, s->bbz, d1, d2,
                                   w.fipx(N), w.fipz(N), w.vx(N), w.vz(N), d3, visco ? w.aux(N) : nullptr, w.p(N),
                                   s->src.p(N), image ? s->img : nullptr, s->img_c);
    nk++;
    *launches += nk;
    if (bad) return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace qp
