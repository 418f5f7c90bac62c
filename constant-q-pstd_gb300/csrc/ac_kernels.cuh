// ac_kernels.cuh -- fused line-pass kernels of the acoustic PSTD step
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
// Each operator is a zero-padded circular convolution done with two
// shared-memory line FFTs (fft_reg.cuh); the multiplier is the Hermitian part
// of the reference's symbol.  Blocks are (TX, L): TX threads per complex line,
// L lines; a z-pass CTA owns 2L consecutive x indices, an x-pass CTA owns 2L
// consecutive z indices.  When a.stage is set, the inputs of the epilogues
// are copied to shared memory asynchronously at kernel start (cp.async), so
// their latency overlaps the FFTs.
#pragma once
#include "fft_reg.cuh"
#include "pass_common.cuh"

namespace qp {

// ---- z pass ----------------------------------------------------------------
// staged fields (each L*2*nzz floats): 0 vz, 1 psi_pz, 2 bbz, 3 psi_vz, 4 Dx
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) ac_zpass_kernel(AcZArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    float2* line = smem + threadIdx.y * ld;
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;  // first x of this thread's line pair
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;
    const size_t fstride = (size_t)L * 2 * nzz;
    float* stg = reinterpret_cast<float*>(smem + (size_t)L * ld) + (size_t)threadIdx.y * 2 * nzz;
    auto S = [&](int f, int row, int k) -> float& { return stg[f * fstride + row * nzz + k]; };
    const float* vz_in = a.vz;
    const float* ppz_in = a.psi_pz;
    const float* bbz_in = a.bbz;
    const float* pvz_in = a.psi_vz;
    const float* dx_in = a.Dx;
    if (a.stage) {
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            for (int h = 0; h < 2; h++) {
                if (!(h ? has1 : has0)) continue;
                const size_t i = (h ? r1 : r0) + k;
                if (a.do_v) {
                    cp_async4(&S(0, h, k), a.vz + i);
                    cp_async4(&S(1, h, k), a.psi_pz + i);
                    cp_async4(&S(2, h, k), a.bbz + i);
                }
                if (a.do_div) {
                    cp_async4(&S(3, h, k), a.psi_vz + i);
                    cp_async4(&S(4, h, k), a.Dx + i);
                }
            }
        }
        cp_async_commit();
    }
    auto rd = [&](int f, const float* g, int h, int k) -> float {
        return a.stage ? S(f, h, k) : g[(h ? r1 : r0) + k];
    };

    if (a.do_v) {
        zload_pair(a.p, line, nzz, has0, has1, r0, r1);
        __syncthreads();
        roundtrip_conv<FP>(smem, ld, fc, L, a.HzP);
        if (a.stage) cp_async_wait_all();
        struct VIn {
            float2 pp, v0, bb;
            float hb, ha;
        };
        batched_for<kEpiBatchZ>(
            threadIdx.x, nzz, blockDim.x,
            [&](int k) {
                VIn r{};
                r.hb = a.h_bz[k];
                r.ha = a.h_az[k];
                if (has0) {
                    r.pp.x = rd(1, ppz_in, 0, k);
                    r.v0.x = rd(0, vz_in, 0, k);
                    r.bb.x = rd(2, bbz_in, 0, k);
                }
                if (has1) {
                    r.pp.y = rd(1, ppz_in, 1, k);
                    r.v0.y = rd(0, vz_in, 1, k);
                    r.bb.y = rd(2, bbz_in, 1, k);
                }
                return r;
            },
            [&](int k, const VIn& r) {
                const float2 d = line[k];
                float2 nv = make_float2(0.f, 0.f);
                if (has0) {
                    const float ps = r.hb * r.pp.x + r.ha * d.x;
                    a.psi_pz[r0 + k] = ps;
                    nv.x = r.v0.x + a.dt * r.bb.x * (d.x + ps);
                    a.vz[r0 + k] = nv.x;
                }
                if (has1) {
                    const float ps = r.hb * r.pp.y + r.ha * d.y;
                    a.psi_pz[r1 + k] = ps;
                    nv.y = r.v0.y + a.dt * r.bb.y * (d.y + ps);
                    a.vz[r1 + k] = nv.y;
                }
                line[k] = nv;
            });
    } else if (a.do_div) {
        zload_pair(a.vz, line, nzz, has0, has1, r0, r1);
    }
    if (!a.do_div) return;
    __syncthreads();
    roundtrip_conv<FP>(smem, ld, fc, L, a.HzM);
    if (a.stage) cp_async_wait_all();
    struct DIn {
        float2 pv, dx;
        float ib, ia;
    };
    batched_for<kEpiBatchZ>(
        threadIdx.x, nzz, blockDim.x,
        [&](int k) {
            DIn r{};
            r.ib = a.i_bz[k];
            r.ia = a.i_az[k];
            if (has0) {
                r.pv.x = rd(3, pvz_in, 0, k);
                r.dx.x = rd(4, dx_in, 0, k);
            }
            if (has1) {
                r.pv.y = rd(3, pvz_in, 1, k);
                r.dx.y = rd(4, dx_in, 1, k);
            }
            return r;
        },
        [&](int k, const DIn& r) {
            const float2 d = line[k];
            float2 dv = make_float2(0.f, 0.f);
            if (has0) {
                const float ps = r.ib * r.pv.x + r.ia * d.x;
                a.psi_vz[r0 + k] = ps;
                dv.x = r.dx.x + (d.x + ps);
                a.div[r0 + k] = dv.x;
            }
            if (has1) {
                const float ps = r.ib * r.pv.y + r.ia * d.y;
                a.psi_vz[r1 + k] = ps;
                dv.y = r.dx.y + (d.y + ps);
                a.div[r1 + k] = dv.y;
            }
            line[k] = dv;
        });
    __syncthreads();
    roundtrip_conv<FP>(smem, ld, fc, L, a.kz2);
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 d = line[k];
        if (has0) a.Lz[r0 + k] = d.x;
        if (has1) a.Lz[r1 + k] = d.y;
    }
}

// ---- x pass ----------------------------------------------------------------
// Staged fields (xstage_fields; each nxx*2L floats, in the (ix, c) walk order,
// only the fields of the pass's mode).  Without the p update, the input of the
// first transform (p, or vx) is its own cp.async group, so the transform starts
// while the epilogue inputs are still arriving.
// P: this launch does the p update (a.do_p); RMAX: largest radix of the plan (12 or 16)
template <bool P, class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) ac_xpass_kernel(AcXArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;
    const XTile T(L, blockIdx.x, nzz, nxx);
    float* sf = reinterpret_cast<float*>(smem);
    float* stg = reinterpret_cast<float*>(smem + (size_t)L * ld);
    const size_t fstride = (size_t)T.tot;
    const unsigned fm = xstage_fields(P, a.do_v, a.do_dx);
    auto S = [&](int f, int g) -> float& { return stg[__popc(fm & ((1u << f) - 1u)) * fstride + g]; };
    if (a.stage) {
        const float* first = a.do_v ? a.p : a.vx;  // the first transform's input when !do_p
        const int ff = a.do_v ? 2 : 6;
        if (!P) {
            for (int g = T.t0; g < T.tot; g += T.nthr) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz < nzz) cp_async4(&S(ff, g), first + (size_t)ix * nzz + iz);
            }
            cp_async_commit();
        }
        for (int g = T.t0; g < T.tot; g += T.nthr) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            if (iz >= nzz) continue;
            const size_t i = (size_t)ix * nzz + iz;
            if (P) {
                cp_async4(&S(1, g), a.Lz + i);
                cp_async4(&S(2, g), a.p + i);
                cp_async4(&S(3, g), a.c1 + i);
                cp_async4(&S(4, g), a.c2 + i);
            }
            if (a.do_v) {
                cp_async4(&S(5, g), a.psi_px + i);
                cp_async4(&S(7, g), a.bbx + i);
            }
            if ((a.do_v || a.do_dx) && (P || ff != 6)) cp_async4(&S(6, g), a.vx + i);
            if (a.do_dx) cp_async4(&S(8, g), a.psi_vx + i);
        }
        cp_async_commit();
    }

    bool have = false;  // smem holds the packed field for the next transform
    if (P) {
        // div feeds the first transform now and the p update later
        batched_for<kEpiBatchX>(
            T.t0, T.tot, T.nthr,
            [&](int g) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                return (iz < nzz) ? a.div[(size_t)ix * nzz + iz] : 0.f;
            },
            [&](int g, float v) {
                int c, ix;
                T.split(g, c, ix);
                sf[T.sidx(c, ix, ld)] = v;
                if (a.stage) S(0, g) = v;
            });
        __syncthreads();
        roundtrip_conv<FP>(smem, ld, fc, L, a.kx2);
        if (a.stage) cp_async_wait_all();
        struct PIn {
            float lz, p0, c1, c2, dv;
        };
        batched_for<kEpiBatchX>(
            T.t0, T.tot, T.nthr,
            [&](int g) {
                PIn r{0.f, 0.f, 0.f, 0.f, 0.f};
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz < nzz) {
                    const size_t i = (size_t)ix * nzz + iz;
                    r.lz = a.stage ? S(1, g) : a.Lz[i];
                    r.p0 = a.stage ? S(2, g) : a.p[i];
                    r.c1 = a.stage ? S(3, g) : a.c1[i];
                    r.c2 = a.stage ? S(4, g) : a.c2[i];
                    r.dv = a.stage ? S(0, g) : a.div[i];
                }
                return r;
            },
            [&](int g, const PIn& r) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                float pn = 0.f;
                if (iz < nzz) {
                    const float lap = sf[T.sidx(c, ix, ld)] + r.lz;
                    pn = r.p0 + r.c1 * (r.dv - r.c2 * lap);
                    if (ix == a.xs && iz == a.zs) pn += a.src;
                }
                sf[T.sidx(c, ix, ld)] = pn;
            });
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
        if (!a.ssg && !a.img) {
            for (int g = T.t0; g < T.tot; g += T.nthr) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz < nzz) a.p[(size_t)ix * nzz + iz] = sf[T.sidx(c, ix, ld)];
            }
        } else {
            // sums of the interior: s, s_c of the illumination and the image
            // and the source wavefield, loaded a group of points at a time
            struct Acc {
                float s, sc, m, mc, ps;
            };
            batched_for<kEpiBatchX>(
                T.t0, T.tot, T.nthr,
                [&](int g) {
                    Acc r{0.f, 0.f, 0.f, 0.f, 0.f};
                    int c, ix;
                    T.split(g, c, ix);
                    const int iz = T.iz0 + c;
                    if (iz < nzz && ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml) {
                        const size_t j = (size_t)(ix - pml) * nz + (iz - pml);
                        if (a.ssg) {
                            r.s = a.ssg[j];
                            r.sc = a.ssg_c[j];
                        }
                        if (a.img) {
                            r.m = a.img[j];
                            r.mc = a.img_c[j];
                            r.ps = a.ps[(size_t)ix * nzz + iz];
                        }
                    }
                    return r;
                },
                [&](int g, const Acc& r) {
                    int c, ix;
                    T.split(g, c, ix);
                    const int iz = T.iz0 + c;
                    if (iz >= nzz) return;
                    const size_t i = (size_t)ix * nzz + iz;
                    const float pn = sf[T.sidx(c, ix, ld)];
                    a.p[i] = pn;
                    if (ix >= pml && ix < nxx - pml && iz >= pml && iz < nzz - pml) {
                        const size_t j = (size_t)(ix - pml) * nz + (iz - pml);
                        if (a.ssg) kahan_add_v(a.ssg, a.ssg_c, j, r.s, r.sc, pn * pn);
                        if (a.img) kahan_add_v(a.img, a.img_c, j, r.m, r.mc, r.ps * pn);
                    }
                });
        }
        have = true;
    }
    if (a.do_v) {
        if (!have) {
            if (a.stage) cp_async_wait_prior();  // p (first group) has landed
            xfill<x_epi_batch<FP>()>(sf, T, ld,
                                     [&](int g, int ix, int iz) { return a.stage ? S(2, g) : a.p[(size_t)ix * nzz + iz]; });
        }
        __syncthreads();
        roundtrip_conv<FP>(smem, ld, fc, L, a.HxP);
        if (a.stage) cp_async_wait_all();
        struct VIn {
            float pp, v0, bb, hb, ha;
        };
        batched_for<x_epi_batch<FP>()>(
            T.t0, T.tot, T.nthr,
            [&](int g) {
                VIn r{0.f, 0.f, 0.f, 0.f, 0.f};
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz < nzz) {
                    const size_t i = (size_t)ix * nzz + iz;
                    r.pp = a.stage ? S(5, g) : a.psi_px[i];
                    r.v0 = a.stage ? S(6, g) : a.vx[i];
                    r.bb = a.stage ? S(7, g) : a.bbx[i];
                    r.hb = a.h_bx[ix];
                    r.ha = a.h_ax[ix];
                }
                return r;
            },
            [&](int g, const VIn& r) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                float nv = 0.f;
                if (iz < nzz) {
                    const size_t i = (size_t)ix * nzz + iz;
                    const float d = sf[T.sidx(c, ix, ld)];
                    const float ps = r.hb * r.pp + r.ha * d;
                    a.psi_px[i] = ps;
                    nv = r.v0 + a.dt * r.bb * (d + ps);
                    a.vx[i] = nv;
                }
                sf[T.sidx(c, ix, ld)] = nv;
            });
        have = true;
    } else {
        have = false;
    }
    if (a.do_dx) {
        if (!have) {
            // vx: the first group without the p update, else in the only group
            if (a.stage) {
                if (P) cp_async_wait_all();
                else cp_async_wait_prior();
            }
            xfill<x_epi_batch<FP>()>(sf, T, ld,
                                     [&](int g, int ix, int iz) { return a.stage ? S(6, g) : a.vx[(size_t)ix * nzz + iz]; });
        }
        __syncthreads();
        roundtrip_conv<FP>(smem, ld, fc, L, a.HxM);
        if (a.stage) cp_async_wait_all();
        struct DIn {
            float pv, ib, ia;
        };
        batched_for<x_epi_batch<FP>()>(
            T.t0, T.tot, T.nthr,
            [&](int g) {
                DIn r{0.f, 0.f, 0.f};
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz < nzz) {
                    r.pv = a.stage ? S(8, g) : a.psi_vx[(size_t)ix * nzz + iz];
                    r.ib = a.i_bx[ix];
                    r.ia = a.i_ax[ix];
                }
                return r;
            },
            [&](int g, const DIn& r) {
                int c, ix;
                T.split(g, c, ix);
                const int iz = T.iz0 + c;
                if (iz >= nzz) return;
                const size_t i = (size_t)ix * nzz + iz;
                const float d = sf[T.sidx(c, ix, ld)];
                const float ps = r.ib * r.pv + r.ia * d;
                a.psi_vx[i] = ps;
                a.Dx[i] = d + ps;
            });
    }
}

}  // namespace qp
