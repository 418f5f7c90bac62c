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
// Blocks are (TX, L): TX threads per complex line, L lines; a z-pass CTA owns
// 2L consecutive x indices, an x-pass CTA owns 2L consecutive z indices.
#include "fft_reg.cuh"
#include "pass_common.cuh"

namespace qp {

// ---- z pass ----------------------------------------------------------------
__global__ void __launch_bounds__(768, 1) ac_zpass_kernel(AcZArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    float2* line = smem + threadIdx.y * ld;
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;  // first x of this thread's line pair
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;

    if (a.do_v) {
        zload_pair(a.p, line, nzz, has0, has1, r0, r1);
        __syncthreads();
        roundtrip_conv(smem, ld, fc, L, a.HzP);
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            const float2 d = line[k];
            const float hb = a.h_bz[k], ha = a.h_az[k];
            float2 nv = make_float2(0.f, 0.f);
            if (has0) {
                const float ps = hb * a.psi_pz[r0 + k] + ha * d.x;
                a.psi_pz[r0 + k] = ps;
                nv.x = a.vz[r0 + k] + a.dt * a.bbz[r0 + k] * (d.x + ps);
                a.vz[r0 + k] = nv.x;
            }
            if (has1) {
                const float ps = hb * a.psi_pz[r1 + k] + ha * d.y;
                a.psi_pz[r1 + k] = ps;
                nv.y = a.vz[r1 + k] + a.dt * a.bbz[r1 + k] * (d.y + ps);
                a.vz[r1 + k] = nv.y;
            }
            line[k] = nv;
        }
    } else if (a.do_div) {
        zload_pair(a.vz, line, nzz, has0, has1, r0, r1);
    }
    if (!a.do_div) return;
    __syncthreads();
    roundtrip_conv(smem, ld, fc, L, a.HzM);
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 d = line[k];
        const float ib = a.i_bz[k], ia = a.i_az[k];
        float2 dv = make_float2(0.f, 0.f);
        if (has0) {
            const float ps = ib * a.psi_vz[r0 + k] + ia * d.x;
            a.psi_vz[r0 + k] = ps;
            dv.x = a.Dx[r0 + k] + (d.x + ps);
            a.div[r0 + k] = dv.x;
        }
        if (has1) {
            const float ps = ib * a.psi_vz[r1 + k] + ia * d.y;
            a.psi_vz[r1 + k] = ps;
            dv.y = a.Dx[r1 + k] + (d.y + ps);
            a.div[r1 + k] = dv.y;
        }
        line[k] = dv;
    }
    __syncthreads();
    roundtrip_conv(smem, ld, fc, L, a.kz2);
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 d = line[k];
        if (has0) a.Lz[r0 + k] = d.x;
        if (has1) a.Lz[r1 + k] = d.y;
    }
}

// ---- x pass ----------------------------------------------------------------
__global__ void __launch_bounds__(768, 1) ac_xpass_kernel(AcXArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    const XTile T(L, blockIdx.x, nzz, nxx);
    float* sf = reinterpret_cast<float*>(smem);

    bool have = false;  // smem holds the packed field for the next transform
    if (a.do_p) {
        xload(a.div, sf, T, ld);
        __syncthreads();
        roundtrip_conv(smem, ld, fc, L, a.kx2);
        for (int g = T.t0; g < T.tot; g += T.nthr) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            float pn = 0.f;
            if (iz < nzz) {
                const size_t i = (size_t)ix * nzz + iz;
                const float lap = sf[T.sidx(c, ix, ld)] + a.Lz[i];
                pn = a.p[i] + a.c1[i] * (a.div[i] - a.c2[i] * lap);
                if (ix == a.xs && iz == a.zs) pn += a.src;
            }
            sf[T.sidx(c, ix, ld)] = pn;
        }
        __syncthreads();
        // receivers of this tile: record (source side) or inject (receiver side)
        if (a.rec_off) {
            const int q0 = a.rec_off[blockIdx.x], q1 = a.rec_off[blockIdx.x + 1];
            for (int q = q0 + T.t0; q < q1; q += T.nthr) {
                const RecEntry e = a.rec[q];
                const int si = T.sidx(e.gz - T.iz0, e.gx, ld);
                if (a.gather_row) a.gather_row[e.ir] = sf[si];
                if (a.obs_row && e.inject) sf[si] = a.obs_row[e.ir];
            }
            __syncthreads();
        }
        const int pml = a.pml, nz = nzz - 2 * pml;
        for (int g = T.t0; g < T.tot; g += T.nthr) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            if (iz >= nzz) continue;
            const size_t i = (size_t)ix * nzz + iz;
            const float pn = sf[T.sidx(c, ix, ld)];
            a.p[i] = pn;
            if (ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml) {
                const size_t j = (size_t)(ix - pml) * nz + (iz - pml);
                if (a.ssg) kahan_add(a.ssg, a.ssg_c, j, pn * pn);
                if (a.img) kahan_add(a.img, a.img_c, j, a.ps[i] * pn);
            }
        }
        have = true;
    }
    if (a.do_v) {
        if (!have) xload(a.p, sf, T, ld);
        __syncthreads();
        roundtrip_conv(smem, ld, fc, L, a.HxP);
        for (int g = T.t0; g < T.tot; g += T.nthr) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            float nv = 0.f;
            if (iz < nzz) {
                const size_t i = (size_t)ix * nzz + iz;
                const float d = sf[T.sidx(c, ix, ld)];
                const float ps = a.h_bx[ix] * a.psi_px[i] + a.h_ax[ix] * d;
                a.psi_px[i] = ps;
                nv = a.vx[i] + a.dt * a.bbx[i] * (d + ps);
                a.vx[i] = nv;
            }
            sf[T.sidx(c, ix, ld)] = nv;
        }
        have = true;
    } else {
        have = false;
    }
    if (a.do_dx) {
        if (!have) xload(a.vx, sf, T, ld);
        __syncthreads();
        roundtrip_conv(smem, ld, fc, L, a.HxM);
        for (int g = T.t0; g < T.tot; g += T.nthr) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            if (iz >= nzz) continue;
            const size_t i = (size_t)ix * nzz + iz;
            const float d = sf[T.sidx(c, ix, ld)];
            const float ps = a.i_bx[ix] * a.psi_vx[i] + a.i_ax[ix] * d;
            a.psi_vx[i] = ps;
            a.Dx[i] = d + ps;
        }
    }
}

void launch_ac_zpass(const AcZArgs& a, cudaStream_t s) {
    const int grid = (a.nxx + 2 * a.L - 1) / (2 * a.L);
    const size_t sm = sizeof(float2) * (size_t)a.L * a.pl.m;
    ac_zpass_kernel<<<grid, dim3(a.pl.tx, a.L), sm, s>>>(a);
}

void launch_ac_xpass(const AcXArgs& a, cudaStream_t s) {
    const int grid = (a.nzz + 2 * a.L - 1) / (2 * a.L);
    const size_t sm = sizeof(float2) * (size_t)a.L * a.pl.m;
    ac_xpass_kernel<<<grid, dim3(a.pl.tx, a.L), sm, s>>>(a);
}

int ac_set_smem_limits() {
    cudaError_t e1 = cudaFuncSetAttribute(ac_zpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaError_t e2 = cudaFuncSetAttribute(ac_xpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return (e1 == cudaSuccess && e2 == cudaSuccess) ? 0 : -1;
}

}  // namespace qp
