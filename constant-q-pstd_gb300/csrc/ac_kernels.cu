// ac_kernels.cu -- fused line-pass kernels of the acoustic PSTD step
// (aps, and both wavefields of artm).
//
// The reference runs one step as 9 cuFFT 2-D C2C transforms and 9 elementwise
// kernels (sgpstd-qmodeling/acps4.cu:517-607).  Every operator in that step is
// separable: the staggered derivatives depend on kx or kz alone and the
// Laplacian symbol is kx^2 + kz^2, so the step here is two passes over HBM:
//   z pass : dz+ p -> CPML -> vz update ; dz- vz -> CPML -> div ; kz^2 part of L
//   x pass : kx^2 part of L -> p update (+ source, receivers, illumination,
//            imaging, Dirichlet injection) ; dx+ p -> CPML -> vx update ;
//            dx- vx -> CPML (x part of the next step's divergence)
// Each derivative is a forward line DFT, a multiply by the Hermitian part of
// the reference's shift symbol, and an inverse line DFT, all in shared memory.
#include "fftline.cuh"

namespace qp {

// ---- z pass ----------------------------------------------------------------
__global__ void __launch_bounds__(256) ac_zpass_kernel(AcZArgs a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    const int ix0 = blockIdx.x * 2 * L;
    const int tot = L * nzz;

    // packed load of a real field: line l <- (ix0+2l, ix0+2l+1)
    auto load = [&](const float* __restrict__ f, float2* dst) {
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int l = g / nzz, k = g - l * nzz;
            const int xa = ix0 + 2 * l;
            float2 v;
            v.x = (xa < nxx) ? f[(size_t)xa * nzz + k] : 0.f;
            v.y = (xa + 1 < nxx) ? f[(size_t)(xa + 1) * nzz + k] : 0.f;
            dst[l * ld + k] = v;
        }
        __syncthreads();
    };

    float2* cur = b0;
    if (a.do_v) {
        load(a.p, b0);
        float2* r = roundtrip_c(b0, b1, L, ld, a.pl, a.HzP);
        float2* o = (r == b0) ? b1 : b0;
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int l = g / nzz, k = g - l * nzz;
            const int xa = ix0 + 2 * l;
            const float2 d = r[l * ld + k];
            const float hb = a.h_bz[k], ha = a.h_az[k];
            float2 nv = make_float2(0.f, 0.f);
            if (xa < nxx) {
                const size_t i = (size_t)xa * nzz + k;
                const float ps = hb * a.psi_pz[i] + ha * d.x;
                a.psi_pz[i] = ps;
                nv.x = a.vz[i] + a.dt * a.bbz[i] * (d.x + ps);
                a.vz[i] = nv.x;
            }
            if (xa + 1 < nxx) {
                const size_t i = (size_t)(xa + 1) * nzz + k;
                const float ps = hb * a.psi_pz[i] + ha * d.y;
                a.psi_pz[i] = ps;
                nv.y = a.vz[i] + a.dt * a.bbz[i] * (d.y + ps);
                a.vz[i] = nv.y;
            }
            o[l * ld + k] = nv;
        }
        __syncthreads();
        cur = o;
    }
    if (!a.do_div) return;
    if (!a.do_v) load(a.vz, b0);
    float2* oth = (cur == b0) ? b1 : b0;
    float2* r = roundtrip_c(cur, oth, L, ld, a.pl, a.HzM);
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
    oth = (o == b0) ? b1 : b0;
    r = roundtrip_r(o, oth, L, ld, a.pl, a.kz2);
    for (int g = threadIdx.x; g < tot; g += blockDim.x) {
        const int l = g / nzz, k = g - l * nzz;
        const int xa = ix0 + 2 * l;
        const float2 d = r[l * ld + k];
        if (xa < nxx) a.Lz[(size_t)xa * nzz + k] = d.x;
        if (xa + 1 < nxx) a.Lz[(size_t)(xa + 1) * nzz + k] = d.y;
    }
}

// ---- x pass ----------------------------------------------------------------
__device__ __forceinline__ void kahan_add(float* s, float* c, size_t i, float v) {
    const float y = v - c[i];
    const float t = s[i] + y;
    c[i] = (t - s[i]) - y;
    s[i] = t;
}

__global__ void __launch_bounds__(256) ac_xpass_kernel(AcXArgs a) {
    extern __shared__ float2 smem[];
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    const int TZ = 2 * L;
    float2* b0 = smem;
    float2* b1 = smem + L * ld;
    const int iz0 = blockIdx.x * TZ;
    const int tot = nxx * TZ;

    // packed load: line l <- columns (iz0+2l, iz0+2l+1), position ix
    auto load = [&](const float* __restrict__ f, float2* dst) {
        float* d = reinterpret_cast<float*>(dst);
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % TZ, ix = g / TZ;
            const int iz = iz0 + c;
            d[2 * ((c >> 1) * ld + ix) + (c & 1)] = (iz < nzz) ? f[(size_t)ix * nzz + iz] : 0.f;
        }
        __syncthreads();
    };
    auto sget = [&](const float2* buf, int c, int ix) -> float {
        return reinterpret_cast<const float*>(buf)[2 * ((c >> 1) * ld + ix) + (c & 1)];
    };
    auto sset = [&](float2* buf, int c, int ix, float v) {
        reinterpret_cast<float*>(buf)[2 * ((c >> 1) * ld + ix) + (c & 1)] = v;
    };

    float2* cur = b0;
    bool have = false;  // cur holds the packed field for the next transform
    if (a.do_p) {
        load(a.div, b0);
        float2* r = roundtrip_r(b0, b1, L, ld, a.pl, a.kx2);
        float2* o = (r == b0) ? b1 : b0;
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % TZ, ix = g / TZ;
            const int iz = iz0 + c;
            float pn = 0.f;
            if (iz < nzz) {
                const size_t i = (size_t)ix * nzz + iz;
                const float lap = sget(r, c, ix) + a.Lz[i];
                pn = a.p[i] + a.c1[i] * (a.div[i] - a.c2[i] * lap);
                if (ix == a.xs && iz == a.zs) pn += a.src;
            }
            sset(o, c, ix, pn);
        }
        __syncthreads();
        // receivers of this tile: record (source side) or inject (receiver side)
        if (a.rec_off) {
            const int r0 = a.rec_off[blockIdx.x], r1 = a.rec_off[blockIdx.x + 1];
            for (int q = r0 + threadIdx.x; q < r1; q += blockDim.x) {
                const RecEntry e = a.rec[q];
                if (a.gather_row) a.gather_row[e.ir] = sget(o, e.gz - iz0, e.gx);
                if (a.obs_row && e.inject) sset(o, e.gz - iz0, e.gx, a.obs_row[e.ir]);
            }
            __syncthreads();
        }
        const int pml = a.pml, nz = nzz - 2 * pml;
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % TZ, ix = g / TZ;
            const int iz = iz0 + c;
            if (iz >= nzz) continue;
            const size_t i = (size_t)ix * nzz + iz;
            const float pn = sget(o, c, ix);
            a.p[i] = pn;
            if (ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml) {
                const size_t j = (size_t)(ix - pml) * nz + (iz - pml);
                if (a.ssg) kahan_add(a.ssg, a.ssg_c, j, pn * pn);
                if (a.img) kahan_add(a.img, a.img_c, j, a.ps[i] * pn);
            }
        }
        cur = o;
        have = true;
    }
    if (a.do_v) {
        if (!have) { load(a.p, b0); cur = b0; }
        float2* oth = (cur == b0) ? b1 : b0;
        float2* r = roundtrip_c(cur, oth, L, ld, a.pl, a.HxP);
        float2* o = (r == b0) ? b1 : b0;
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % TZ, ix = g / TZ;
            const int iz = iz0 + c;
            float nv = 0.f;
            if (iz < nzz) {
                const size_t i = (size_t)ix * nzz + iz;
                const float d = sget(r, c, ix);
                const float ps = a.h_bx[ix] * a.psi_px[i] + a.h_ax[ix] * d;
                a.psi_px[i] = ps;
                nv = a.vx[i] + a.dt * a.bbx[i] * (d + ps);
                a.vx[i] = nv;
            }
            sset(o, c, ix, nv);
        }
        __syncthreads();
        cur = o;
        have = true;
    } else {
        have = false;
    }
    if (a.do_dx) {
        if (!have) { load(a.vx, b0); cur = b0; }
        float2* oth = (cur == b0) ? b1 : b0;
        float2* r = roundtrip_c(cur, oth, L, ld, a.pl, a.HxM);
        for (int g = threadIdx.x; g < tot; g += blockDim.x) {
            const int c = g % TZ, ix = g / TZ;
            const int iz = iz0 + c;
            if (iz >= nzz) continue;
            const size_t i = (size_t)ix * nzz + iz;
            const float d = sget(r, c, ix);
            const float ps = a.i_bx[ix] * a.psi_vx[i] + a.i_ax[ix] * d;
            a.psi_vx[i] = ps;
            a.Dx[i] = d + ps;
        }
    }
}

void launch_ac_zpass(const AcZArgs& a, cudaStream_t s) {
    const int grid = (a.nxx + 2 * a.L - 1) / (2 * a.L);
    const size_t sm = sizeof(float2) * 2 * (size_t)a.L * a.pl.m;
    ac_zpass_kernel<<<grid, 256, sm, s>>>(a);
}

void launch_ac_xpass(const AcXArgs& a, cudaStream_t s) {
    const int grid = (a.nzz + 2 * a.L - 1) / (2 * a.L);
    const size_t sm = sizeof(float2) * 2 * (size_t)a.L * a.pl.m;
    ac_xpass_kernel<<<grid, 256, sm, s>>>(a);
}

int ac_set_smem_limits() {
    cudaError_t e1 = cudaFuncSetAttribute(ac_zpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaError_t e2 = cudaFuncSetAttribute(ac_xpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return (e1 == cudaSuccess && e2 == cudaSuccess) ? 0 : -1;
}

}  // namespace qp
