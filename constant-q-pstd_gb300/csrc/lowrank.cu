// lowrank.cu -- the low-rank form of the constant-Q symbol on the device, and
// its C ABI.
//
// The reference defines the form (sgpstd-qmodeling/sglowrank.c) and the
// kernels that apply it (sgpstd-qmodeling/acsglw.cu:1375-1497: multv_kernel
// multiplies the 2-D spectrum by V_b / N for each of the row factors, an
// inverse 2-D FFT per factor, sumlw_kernel forms pst_a = sum_b A[a][b] q_b in
// double, sumlw2_kernel forms out = sum_a U[x][a] pst_a), but its call sites
// are commented out (acsglw.cu:367-389), so no time step uses it.  Here the
// operator out = sum_b c_b(x) Re F^-1[Vt_b F in] / N, c_b(x) = sum_a U[x][a]
// A[a][b] (formed once in FP64), is three fused passes over the half spectra
// in kz (as the other constant-Q operators):
//   z pass      : real z-lines (two per complex line) -> half spectrum G
//   x pass      : per kz column and factor b, the forward x transform, the
//                 multiply by V_b (mirrored, the reference's consist_Vt,
//                 sglowrank.c:103-145) and the inverse x transform
//   z pass      : per factor b (one launch each), the inverse z transform,
//                 accumulated with the point weights c_b(x) in the epilogue,
//                 so the k-space and x-space factors meet inside the FFT
//                 passes and only the output field is written.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/qpstd.h"
#include "fft_reg.cuh"
#include "host_setup.h"
#include "lowrank.h"
#include "pass_common.cuh"

namespace qp {
void set_last_error(const std::string& m);

__global__ void __launch_bounds__(768, 1) lr_zfwd_kernel(LrZArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx, nzh = a.nzh;
    float2* line = smem + threadIdx.y * ld;
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;
    zload_pair(a.in, line, nzz, has0, has1, r0, r1);
    __syncthreads();
    dft_n<-1>(smem, ld, fc, L);
    zunpack(line, a.spec, nzz, nzh, has0, has1, xa);
}

// L kz columns per CTA (L a power of two), factor b = blockIdx.y: the forward
// x transform is repeated per factor (one factor per CTA keeps the pass free
// of register spills, which a factor loop around the transforms is not).
__global__ void __launch_bounds__(768, 1) lr_xspec_kernel(LrXArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nxx = a.nxx, nzh = a.nzh, nxh = a.nxh;
    const int lg = 31 - __clz(L);
    const int kz0 = blockIdx.x * L, b = blockIdx.y;
    const int t0 = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    const int tot = L * nxx;
    float2* line = smem + threadIdx.y * ld;
    for (int g = t0; g < tot; g += nthr) {
        const int c = g & (L - 1), ix = g >> lg;
        const int kz = kz0 + c;
        smem[c * ld + ix] = (kz < nzh) ? a.in[(size_t)ix * nzh + kz] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    dft_n<-1>(smem, ld, fc, L);
    const int kz = min(kz0 + (int)threadIdx.y, nzh - 1);
    const float* Vb = a.V + (size_t)b * nxh * nzh;
    for (int ix = threadIdx.x; ix < nxx; ix += blockDim.x) {
        const int ih = (ix < nxh) ? ix : nxx - ix;
        line[ix] = cscale(line[ix], __ldg(&Vb[(size_t)ih * nzh + kz]) * a.norm);
    }
    __syncthreads();
    dft_n<+1>(smem, ld, fc, L);
    float2* out = a.out + (size_t)b * nxx * nzh;
    for (int g = t0; g < tot; g += nthr) {
        const int c = g & (L - 1), ix = g >> lg;
        if (kz0 + c < nzh) out[(size_t)ix * nzh + kz0 + c] = smem[c * ld + ix];
    }
}

// Factor b: out (+)= c_b(x) q_b(x), q_b the inverse z transform of half
// spectrum b (the first factor overwrites out, the others accumulate).
__global__ void __launch_bounds__(768, 1) lr_zinv_kernel(LrZArgs a, int b) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx, nzh = a.nzh;
    float2* line = smem + threadIdx.y * ld;
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;
    zrepack(a.spec + (size_t)b * nxx * nzh, line, nzz, nzh, has0, has1, xa);
    __syncthreads();
    dft_n<+1>(smem, ld, fc, L);
    const float* cb = a.c + (size_t)b * nxx * nzz;
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 v = line[k];
        if (has0) a.out[r0 + k] = fmaf(__ldg(&cb[r0 + k]), v.x, b ? a.out[r0 + k] : 0.f);
        if (has1) a.out[r1 + k] = fmaf(__ldg(&cb[r1 + k]), v.y, b ? a.out[r1 + k] : 0.f);
    }
}

static size_t lsm(int L, int m) { return sizeof(float2) * (size_t)L * m; }

void launch_lr_zfwd(const LrZArgs& a, cudaStream_t s) {
    lr_zfwd_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), dim3(a.pl.tx, a.L), lsm(a.L, a.pl.m), s>>>(a);
}
void launch_lr_xspec(const LrXArgs& a, cudaStream_t s) {
    lr_xspec_kernel<<<dim3((a.nzh + a.L - 1) / a.L, a.row), dim3(a.pl.tx, a.L), lsm(a.L, a.pl.m), s>>>(a);
}
void launch_lr_zinv(const LrZArgs& a, cudaStream_t s) {
    for (int b = 0; b < a.row; b++)
        lr_zinv_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), dim3(a.pl.tx, a.L), lsm(a.L, a.pl.m), s>>>(a, b);
}
int lr_set_smem_limits() {
    const int lim = 200 * 1024;
    int bad = cudaFuncSetAttribute(lr_zfwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(lr_xspec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(lr_zinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    return bad ? -1 : 0;
}

}  // namespace qp

using namespace qp;

// ---- C ABI ------------------------------------------------------------------------
struct qpstd_lowrank {
    int nxx = 0, nzz = 0, nzh = 0, nxh = 0, row = 0;
    cudaStream_t stream = nullptr;
    FFTPlanDev px{}, pz{};
    int Lz = 1, Lx = 1;
    std::vector<void*> allocs;
    float *V = nullptr, *c = nullptr, *in = nullptr, *out = nullptr;
    float2 *G = nullptr, *Q = nullptr;
};

namespace {

int lr_fail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

int lr_cuda(cudaError_t e, const char* where) {
    return lr_fail(e == cudaErrorMemoryAllocation ? QPSTD_ENOMEM : QPSTD_ECUDA,
                   std::string(where) + ": " + cudaGetErrorString(e));
}

template <class T> int lr_alloc(qpstd_lowrank* h, T** p, size_t n) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * std::max<size_t>(n, 1));
    if (e != cudaSuccess) return lr_cuda(e, "cudaMalloc");
    h->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return QPSTD_OK;
}

int lr_plan(qpstd_lowrank* h, int n, FFTPlanDev& d) {
    HostPlan hp;
    if (build_plan_host(n, hp)) return lr_fail(QPSTD_ENOTSUP, "no FFT plan for this length");
    if (fill_plan_dev(hp, d)) return lr_fail(QPSTD_ENOTSUP, "transform needs more threads per line than a CTA holds");
    std::vector<float2> t;
    plan_tables(hp, t);
    float2* p = nullptr;
    int rc = lr_alloc(h, &p, t.size());
    if (rc) return rc;
    const cudaError_t e = cudaMemcpy(p, t.data(), sizeof(float2) * t.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return lr_cuda(e, "upload");
    d.w = p;
    d.chirp = hp.blue ? p + hp.w.size() : nullptr;
    d.bhat = hp.blue ? p + hp.w.size() + hp.chirp.size() : nullptr;
    return QPSTD_OK;
}

int lr_sizes_ok(int nxx, int nzz, int row, int col) {
    if (nxx < 2 || nzz < 2 || row < 1 || col < 1 || row > 64 || col > 64)
        return lr_fail(QPSTD_EINVAL, "bad low-rank sizes (grid >= 2 x 2, 1 <= row, col <= 64)");
    if ((long long)nxx * nzz > (1ll << 30)) return lr_fail(QPSTD_EINVAL, "grid too large");
    return QPSTD_OK;
}

}  // namespace

extern "C" int qpstd_lowrank_decompose(int nxx, int nzz, float dx, float dz, float dt, const float* vp,
                                       const float* tao, const float* gam, int row, int col,
                                       unsigned long long seed, float* U, float* V, double* A, int* jrr, int* irr) {
    int rc = lr_sizes_ok(nxx, nzz, row, col);
    if (rc) return rc;
    if (!vp || !tao || !gam) return lr_fail(QPSTD_EINVAL, "null model pointer");
    LowRankFactors f;
    lowrank_decompose(nxx, nzz, dx, dz, dt, vp, tao, gam, row, col, seed, f);
    if (U) std::copy(f.U.begin(), f.U.end(), U);
    if (V) std::copy(f.V.begin(), f.V.end(), V);
    if (A) std::copy(f.A.begin(), f.A.end(), A);
    if (jrr) std::copy(f.jrr.begin(), f.jrr.end(), jrr);
    if (irr) std::copy(f.irr.begin(), f.irr.end(), irr);
    return QPSTD_OK;
}

extern "C" int qpstd_lowrank_check(int nxx, int nzz, float dx, float dz, float dt, int row, int col, const float* U,
                                   const double* A, const float* V, const float* vp, const float* tao,
                                   const float* gam, int is, float* We, float* Wa) {
    int rc = lr_sizes_ok(nxx, nzz, row, col);
    if (rc) return rc;
    if (!U || !A || !V || !vp || !tao || !gam || !We || !Wa) return lr_fail(QPSTD_EINVAL, "null pointer");
    if (is < 0 || is >= nxx * nzz) return lr_fail(QPSTD_EINVAL, "point index outside the grid");
    std::vector<double> k;
    lowrank_khalf(nxx, nzz, dx, dz, k);
    const size_t N2 = k.size();
    std::vector<double> tp(row, 0.0);
    for (int b = 0; b < row; b++)
        for (int a = 0; a < col; a++) tp[b] += (double)U[(size_t)is * col + a] * A[(size_t)a * row + b];
    for (size_t j = 0; j < N2; j++) {
        We[j] = (float)lowrank_symbol(vp[is], gam[is], tao[is], dt, k[j]);
        double s = 0.0;
        for (int b = 0; b < row; b++) s += tp[b] * V[(size_t)b * N2 + j];
        Wa[j] = (float)s;
    }
    return QPSTD_OK;
}

extern "C" int qpstd_lowrank_create(int nxx, int nzz, int row, int col, const float* U, const float* V,
                                    const double* A, qpstd_lowrank** out) {
    if (!out) return lr_fail(QPSTD_EINVAL, "null output handle");
    *out = nullptr;
    int rc = lr_sizes_ok(nxx, nzz, row, col);
    if (rc) return rc;
    if (!U || !V || !A) return lr_fail(QPSTD_EINVAL, "null factor");
    if (lr_set_smem_limits()) return lr_fail(QPSTD_ECUDA, "cannot raise the shared-memory limit of the passes");
    qpstd_lowrank* h = new qpstd_lowrank();
    h->nxx = nxx;
    h->nzz = nzz;
    h->nzh = nzz / 2 + 1;
    h->nxh = nxx / 2 + 1;
    h->row = row;
    auto bail = [&](int code) {
        qpstd_lowrank_destroy(h);
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(lr_cuda(e, "cudaStreamCreate"));
    if ((rc = lr_plan(h, nxx, h->px)) || (rc = lr_plan(h, nzz, h->pz))) return bail(rc);
    if (8.0 * std::max(h->px.m, h->pz.m) > 200 * 1024) return bail(lr_fail(QPSTD_ENOTSUP, "line too long for one CTA"));
    const size_t N1 = (size_t)nxx * nzz, N2 = (size_t)h->nxh * h->nzh, NS = (size_t)nxx * h->nzh;
    if ((rc = lr_alloc(h, &h->V, (size_t)row * N2)) || (rc = lr_alloc(h, &h->c, (size_t)row * N1)) ||
        (rc = lr_alloc(h, &h->in, N1)) || (rc = lr_alloc(h, &h->out, N1)) || (rc = lr_alloc(h, &h->G, NS)) ||
        (rc = lr_alloc(h, &h->Q, (size_t)row * NS)))
        return bail(rc);
    // point weights c_b(x) = sum_a U[x][a] A[a][b], formed in FP64, stored factor-major
    std::vector<float> c((size_t)row * N1);
    for (size_t x = 0; x < N1; x++)
        for (int b = 0; b < row; b++) {
            double s = 0.0;
            for (int a = 0; a < col; a++) s += (double)U[x * col + a] * A[(size_t)a * row + b];
            c[(size_t)b * N1 + x] = (float)s;
        }
    if ((e = cudaMemcpy(h->c, c.data(), sizeof(float) * c.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(h->V, V, sizeof(float) * (size_t)row * N2, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(lr_cuda(e, "upload"));
    const int pairs = (nxx + 1) / 2;
    h->Lz = choose_L(pairs, h->pz.m, h->pz.tx, 1, false);
    h->Lx = choose_L(h->nzh, h->px.m, h->px.tx, 1, true);
    *out = h;
    return QPSTD_OK;
}

extern "C" int qpstd_lowrank_destroy(qpstd_lowrank* h) {
    if (!h) return QPSTD_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void* p : h->allocs) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return QPSTD_OK;
}

extern "C" int qpstd_lowrank_apply_device(qpstd_lowrank* h, const float* d_in, float* d_out, void* stream) {
    if (!h || !d_in || !d_out) return lr_fail(QPSTD_EINVAL, "null argument");
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    LrZArgs z{};
    z.nxx = h->nxx; z.nzz = h->nzz; z.nzh = h->nzh; z.row = h->row; z.pl = h->pz;
    z.L = h->Lz; z.in = d_in; z.spec = h->G;
    launch_lr_zfwd(z, st);
    LrXArgs x{};
    x.nxx = h->nxx; x.nzz = h->nzz; x.nzh = h->nzh; x.nxh = h->nxh; x.L = h->Lx; x.row = h->row; x.pl = h->px;
    x.V = h->V; x.in = h->G; x.out = h->Q; x.norm = (float)(1.0 / ((double)h->nxx * h->nzz));
    launch_lr_xspec(x, st);
    z.in = nullptr; z.spec = h->Q; z.c = h->c; z.out = d_out;
    launch_lr_zinv(z, st);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lr_cuda(e, "kernel launch");
    return QPSTD_OK;
}

extern "C" int qpstd_lowrank_apply(qpstd_lowrank* h, const float* in, float* out) {
    if (!h || !in || !out) return lr_fail(QPSTD_EINVAL, "null argument");
    const size_t bytes = sizeof(float) * (size_t)h->nxx * h->nzz;
    cudaError_t e = cudaMemcpyAsync(h->in, in, bytes, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return lr_cuda(e, "upload");
    const int rc = qpstd_lowrank_apply_device(h, h->in, h->out, h->stream);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, h->out, bytes, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return lr_cuda(e, "download");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return lr_cuda(e, "apply");
    return QPSTD_OK;
}
