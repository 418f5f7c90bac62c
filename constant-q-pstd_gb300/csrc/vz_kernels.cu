// vz_kernels.cu -- fused passes of the constant-Q (vaps / qrtm) step.
//
// Reference step (sgpstd-qmodeling/acsglw.cu:511-645, sgpstd-qrtm/acsglw.cu:511-657):
//   div   = dx- vx + dz- vz (+ CPML)
//   Y2,Y3,Y4 = F^-1[(k^2)^(1/32), k^2, (k^2)^(33/32) . F div]       (3 inverse 2-D FFTs)
//   total = (1-32g) div + 32g vwd Y2 - dt^2 vp^2 lam/12 ((1-64g) Y3 + 64g vwd Y4)
//   D     = F^-1[(k^2)^0.505 F total]
//   p    += rho vp^2 dt lam (total -/+ dt tau D/2) -/+ dt tau aux     (vaps / qrtm)
//   Px,Pz = staggered gradients of p (+ CPML), v update
//   aux   = F^-1[(k^2)^0.505 F p]  (vaps)  or the stabilised filter S(k,t) (qrtm)
// Here: z pass A (div, z-FFT), x-spectral pass (3 symbols), z pass B (total,
// z-FFT), x-spectral pass (k^0.505), z pass C (D, p update, z-FFT of p, Pz and
// vz update), x pass (Px, vx update, next Dx; shared with the acoustic step),
// x-spectral pass (aux symbol).  The aux spectrum is turned back into a real
// field at the start of the next step's z pass A.
#include "fftline.cuh"

namespace qp {

__device__ __forceinline__ void kahan_add2(float* s, float* c, size_t i, float v) {
    const float y = v - c[i];
    const float t = s[i] + y;
    c[i] = (t - s[i]) - y;
    s[i] = t;
}

// packed load of two real z-lines per complex line
__device__ __forceinline__ void zload(const float* __restrict__ f, float2* dst, int L, int ld, int nxx, int nzz,
                                      int ix0) {
    const int tot = L * nzz;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        float2 v;
        v.x = (xa < nxx) ? f[(size_t)xa * nzz + k] : 0.f;
        v.y = (xa + 1 < nxx) ? f[(size_t)(xa + 1) * nzz + k] : 0.f;
        dst[l * ld + k] = v;
    }
    __syncthreads();
}

// Full packed spectrum Z = A + iB of lines (xa, xa+1) from their half spectra.
__device__ __forceinline__ void zrepack(const float2* __restrict__ S, float2* dst, int L, int ld, int nxx, int nzz,
                                        int nzh, int ix0) {
    const int tot = L * nzz;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const int kk = (k < nzh) ? k : nzz - k;
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
        if (xa < nxx) A = S[(size_t)xa * nzh + kk];
        if (xa + 1 < nxx) B = S[(size_t)(xa + 1) * nzh + kk];
        float2 z;
        if (k < nzh) z = make_float2(A.x - B.y, A.y + B.x);
        else z = make_float2(A.x + B.y, -A.y + B.x);
        dst[l * ld + k] = z;
    }
    __syncthreads();
}

// Split a packed forward spectrum into the half spectra of its two lines.
__device__ __forceinline__ void zunpack(const float2* r, float2* __restrict__ S, int L, int ld, int nxx, int nzz,
                                        int nzh, int ix0) {
    const int tot = L * nzh;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzh, k = g - l * nzh;
        const int xa = ix0 + 2 * l;
        const float2 z = r[l * ld + k];
        const float2 w = r[l * ld + ((k == 0) ? 0 : nzz - k)];
        if (xa < nxx) S[(size_t)xa * nzh + k] = make_float2(0.5f * (z.x + w.x), 0.5f * (z.y - w.y));
        if (xa + 1 < nxx) S[(size_t)(xa + 1) * nzh + k] = make_float2(0.5f * (z.y + w.y), -0.5f * (z.x - w.x));
    }
}

// ---- z pass A ---------------------------------------------------------------
__global__ void __launch_bounds__(256) vz_passA_kernel(VzArgsA a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx, nzh = a.nzh;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    const int ix0 = blockIdx.x * 2 * L;
    const int tot = L * nzz;
    if (a.aux_spec) {
        zrepack(a.aux_spec, b0, L, ld, nxx, nzz, nzh, ix0);
        float2* r = dft_lines(b0, b1, L, ld, a.pl, +1.f);
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int l = g / nzz, k = g - l * nzz;
            const int xa = ix0 + 2 * l;
            const float2 v = r[l * ld + k];
            if (xa < nxx) a.aux[(size_t)xa * nzz + k] = v.x;
            if (xa + 1 < nxx) a.aux[(size_t)(xa + 1) * nzz + k] = v.y;
        }
        __syncthreads();
    }
    zload(a.vz, b0, L, ld, nxx, nzz, ix0);
    float2* r = roundtrip_c(b0, b1, L, ld, a.pl, a.HzM);
    float2* o = (r == b0) ? b1 : b0;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 d = r[l * ld + k];
        const float ib = a.i_bz[k], ia = a.i_az[k];
        float2 dv = make_float2(0.f, 0.f);
        if (xa < nxx) {
            const size_t i = (size_t)xa * nzz + k;
            const float ps = ib * a.psi_vz[i] + ia * d.x;
            a.psi_vz[i] = ps;
            dv.x = a.Dx[i] + (d.x + ps);
            a.div[i] = dv.x;
        }
        if (xa + 1 < nxx) {
            const size_t i = (size_t)(xa + 1) * nzz + k;
            const float ps = ib * a.psi_vz[i] + ia * d.y;
            a.psi_vz[i] = ps;
            dv.y = a.Dx[i] + (d.y + ps);
            a.div[i] = dv.y;
        }
        o[l * ld + k] = dv;
    }
    __syncthreads();
    float2* oth = (o == b0) ? b1 : b0;
    r = dft_lines(o, oth, L, ld, a.pl, -1.f);
    zunpack(r, a.G, L, ld, nxx, nzz, nzh, ix0);
}

// ---- x-spectral pass ----------------------------------------------------------
__global__ void __launch_bounds__(256) vz_xspec_kernel(VxsArgs a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nxx = a.nxx, nzh = a.nzh;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    float2* b2 = smem + 2 * L * ld;  // mode 0 keeps the forward spectrum here
    const int kz0 = blockIdx.x * L;
    const int tot = L * nxx;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int c = g % L, ix = g / L;
        const int kz = kz0 + c;
        b0[c * ld + ix] = (kz < nzh) ? a.in[(size_t)ix * nzh + kz] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2* X = dft_lines(b0, b1, L, ld, a.pl, -1.f);
    const int nout = (a.mode == 0) ? 3 : 1;
    if (nout == 3 && X != b2) {
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g / nxx, ix = g - c * nxx;
            b2[c * ld + ix] = X[c * ld + ix];
        }
        __syncthreads();
        X = b2;
    }
    for (int j = 0; j < nout; j++) {
        // three outputs: X stays in b2 and each output ping-pongs in b0/b1;
        // one output: the product goes to the free buffer, X's buffer is scratch
        float2* y = (nout == 3) ? b0 : ((X == b0) ? b1 : b0);
        float2* z = (nout == 3) ? b1 : X;
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g / nxx, ix = g - c * nxx;
            const int kz = kz0 + c;
            const float k2 = a.kx2[ix] + a.kz2[(kz < nzh) ? kz : 0];
            float sym;
            if (a.mode == 0) {
                if (j == 1) {
                    sym = k2;
                } else {
                    const float lk = log2f(k2);
                    const float k32 = exp2f(lk * (1.f / 32.f));
                    sym = (j == 0) ? k32 : k2 * k32;
                }
            } else {
                const float ka = exp2f(0.505f * log2f(k2));
                if (a.mode == 1) {
                    sym = ka;
                } else {
                    const float num = 2.f * a.eta6 * ka * (1.f + a.tao * a.dt * ka);
                    const float den = expf(-a.tao * a.tt * ka) + a.eta6 * expf(a.tao * a.dt * ka);
                    sym = ka - num / den;
                }
            }
            y[c * ld + ix] = cscale(X[c * ld + ix], sym * a.norm);
        }
        __syncthreads();
        float2* r = dft_lines(y, z, L, ld, a.pl, +1.f);
        float2* out = (j == 0) ? a.out0 : ((j == 1) ? a.out1 : a.out2);
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % L, ix = g / L;
            const int kz = kz0 + c;
            if (kz < nzh) out[(size_t)ix * nzh + kz] = r[c * ld + ix];
        }
        __syncthreads();
    }
}

// ---- z pass B -----------------------------------------------------------------
__global__ void __launch_bounds__(256) vz_passB_kernel(VzArgsB a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx, nzh = a.nzh;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    float2* acc = smem + 2 * L * ld;  // running total (packed pairs)
    const int ix0 = blockIdx.x * 2 * L;
    const int tot = L * nzz;
    const float2* specs[3] = {a.Y2, a.Y3, a.Y4};
    for (int j = 0; j < 3; j++) {
        zrepack(specs[j], b0, L, ld, nxx, nzz, nzh, ix0);
        float2* r = dft_lines(b0, b1, L, ld, a.pl, +1.f);
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int l = g / nzz, k = g - l * nzz;
            const int xa = ix0 + 2 * l;
            const float2 y = r[l * ld + k];
            float2 t = (j == 0) ? make_float2(0.f, 0.f) : acc[l * ld + k];
            const float* cf = (j == 0) ? a.y2 : ((j == 1) ? a.y3c : a.y4c);
            const float sg = (j == 0) ? 1.f : -1.f;
            if (xa < nxx) t.x += sg * cf[(size_t)xa * nzz + k] * y.x;
            if (xa + 1 < nxx) t.y += sg * cf[(size_t)(xa + 1) * nzz + k] * y.y;
            acc[l * ld + k] = t;
        }
        __syncthreads();
    }
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        float2 t = acc[l * ld + k];
        float2 v = make_float2(0.f, 0.f);
        if (xa < nxx) {
            const size_t i = (size_t)xa * nzz + k;
            v.x = a.y1[i] * a.div[i] + t.x;
            a.total[i] = v.x;
        }
        if (xa + 1 < nxx) {
            const size_t i = (size_t)(xa + 1) * nzz + k;
            v.y = a.y1[i] * a.div[i] + t.y;
            a.total[i] = v.y;
        }
        b0[l * ld + k] = v;
    }
    __syncthreads();
    float2* r = dft_lines(b0, b1, L, ld, a.pl, -1.f);
    zunpack(r, a.T, L, ld, nxx, nzz, nzh, ix0);
}

// ---- z pass C -----------------------------------------------------------------
__global__ void __launch_bounds__(256) vz_passC_kernel(VzArgsC a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx, nzh = a.nzh;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    const int ix0 = blockIdx.x * 2 * L;
    const int tot = L * nzz;
    zrepack(a.Dspec, b0, L, ld, nxx, nzz, nzh, ix0);
    float2* r = dft_lines(b0, b1, L, ld, a.pl, +1.f);
    float2* o = (r == b0) ? b1 : b0;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 D = r[l * ld + k];
        float2 pn = make_float2(0.f, 0.f);
        if (xa < nxx) {
            const size_t i = (size_t)xa * nzz + k;
            pn.x = a.p[i] + a.e1[i] * (a.total[i] + a.sgn * a.e2[i] * D.x) + a.sgn * a.e3[i] * a.aux[i];
            if (xa == a.xs && k == a.zs) pn.x += a.src;
        }
        if (xa + 1 < nxx) {
            const size_t i = (size_t)(xa + 1) * nzz + k;
            pn.y = a.p[i] + a.e1[i] * (a.total[i] + a.sgn * a.e2[i] * D.y) + a.sgn * a.e3[i] * a.aux[i];
            if (xa + 1 == a.xs && k == a.zs) pn.y += a.src;
        }
        o[l * ld + k] = pn;
    }
    __syncthreads();
    if (a.rec_off) {
        float* of = reinterpret_cast<float*>(o);
        const int r0 = a.rec_off[blockIdx.x], r1 = a.rec_off[blockIdx.x + 1];
        for (int q = r0 + threadIdx.x; q < r1; q += blockDim.x) {
            const RecEntry e = a.rec[q];
            const int rel = e.gx - ix0;
            const size_t si = 2 * ((size_t)(rel >> 1) * ld + e.gz) + (rel & 1);
            if (a.gather_row) a.gather_row[e.ir] = of[si];
            if (a.obs_row && e.inject) of[si] = a.obs_row[e.ir];
        }
        __syncthreads();
    }
    const int pml = a.pml, nz = nzz - 2 * pml;
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 pn = o[l * ld + k];
        for (int h = 0; h < 2; h++) {
            const int ix = xa + h;
            if (ix >= nxx) break;
            const float v = h ? pn.y : pn.x;
            const size_t i = (size_t)ix * nzz + k;
            a.p[i] = v;
            if (ix >= pml && ix < nxx - pml && k >= pml && k < nzz - pml) {
                const size_t j = (size_t)(ix - pml) * nz + (k - pml);
                if (a.ssg) kahan_add2(a.ssg, a.ssg_c, j, v * v);
                if (a.img) kahan_add2(a.img, a.img_c, j, a.ps[i] * v);
            }
        }
    }
    // forward z transform of the new p: half spectrum for the aux operator and
    // the staggered z derivative from the same transform
    float2* oth = (o == b0) ? b1 : b0;
    float2* X = dft_lines(o, oth, L, ld, a.pl, -1.f);
    zunpack(X, a.P, L, ld, nxx, nzz, nzh, ix0);
    __syncthreads();
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        X[l * ld + k] = cmul(X[l * ld + k], __ldg(&a.HzP[k]));
    }
    __syncthreads();
    oth = (X == b0) ? b1 : b0;
    r = dft_lines(X, oth, L, ld, a.pl, +1.f);
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 d = r[l * ld + k];
        const float hb = a.h_bz[k], ha = a.h_az[k];
        if (xa < nxx) {
            const size_t i = (size_t)xa * nzz + k;
            const float ps = hb * a.psi_pz[i] + ha * d.x;
            a.psi_pz[i] = ps;
            a.vz[i] = a.vz[i] + a.dt * a.bbz[i] * (d.x + ps);
        }
        if (xa + 1 < nxx) {
            const size_t i = (size_t)(xa + 1) * nzz + k;
            const float ps = hb * a.psi_pz[i] + ha * d.y;
            a.psi_pz[i] = ps;
            a.vz[i] = a.vz[i] + a.dt * a.bbz[i] * (d.y + ps);
        }
    }
}

// ---- z inverse only -------------------------------------------------------------
__global__ void __launch_bounds__(256) vz_zinv_kernel(VzArgsI a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    const int ix0 = blockIdx.x * 2 * L;
    zrepack(a.spec, b0, L, ld, nxx, nzz, a.nzh, ix0);
    float2* r = dft_lines(b0, b1, L, ld, a.pl, +1.f);
    for (int g = threadIdx.x; g < L * nzz; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 v = r[l * ld + k];
        if (xa < nxx) a.out[(size_t)xa * nzz + k] = v.x;
        if (xa + 1 < nxx) a.out[(size_t)(xa + 1) * nzz + k] = v.y;
    }
}

// ---- launchers -------------------------------------------------------------------
static size_t zsm(int L, int m, int nbuf) { return sizeof(float2) * (size_t)nbuf * L * m; }

void launch_vz_passA(const VzArgsA& a, cudaStream_t s) {
    vz_passA_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), 256, zsm(a.L, a.pl.m, 2), s>>>(a);
}
void launch_vz_xspec(const VxsArgs& a, cudaStream_t s) {
    vz_xspec_kernel<<<(a.nzh + a.L - 1) / a.L, 256, zsm(a.L, a.pl.m, a.mode == 0 ? 3 : 2), s>>>(a);
}
void launch_vz_passB(const VzArgsB& a, cudaStream_t s) {
    vz_passB_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), 256, zsm(a.L, a.pl.m, 3), s>>>(a);
}
void launch_vz_passC(const VzArgsC& a, cudaStream_t s) {
    vz_passC_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), 256, zsm(a.L, a.pl.m, 2), s>>>(a);
}
void launch_vz_zinv(const VzArgsI& a, cudaStream_t s) {
    vz_zinv_kernel<<<(a.nxx + 2 * a.L - 1) / (2 * a.L), 256, zsm(a.L, a.pl.m, 2), s>>>(a);
}

int vz_set_smem_limits() {
    int bad = 0;
    bad |= cudaFuncSetAttribute(vz_passA_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_passB_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_passC_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_zinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess;
    return bad ? -1 : 0;
}

}  // namespace qp
