// vz_kernels.cuh -- fused passes of the constant-Q (vaps / qrtm) step.
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
//
// Half spectra: S[ix*nzh + kz], kz in [0, nzz/2].  Two real z-lines a, b are
// transformed as one complex line z = a + ib; A(k) = (Z(k) + conj Z(n-k))/2,
// B(k) = (Z(k) - conj Z(n-k))/(2i), and back Z(k) = A(k) + iB(k).
#pragma once
#include "fft_reg.cuh"
#include "pass_common.cuh"

namespace qp {

// this thread's packed line <- the inverse z transform of the half spectra S
// of rows (xa, xa+1).  The caller has synchronised since the line was last
// read; ends with a barrier.  With a compiled plan that is not Bluestein the
// repacking is the first pass's load (no sweep through shared memory first).
template <class FP>
__device__ __forceinline__ void zrepack_inverse(const float2* __restrict__ S, float2* smem, int ld, const FFTCtx& fc,
                                                int L, int nzz, int nzh, bool has0, bool has1, int xa) {
    if constexpr (FP::kCompiled) {
        if (!fc.blue) {
            FP::template run_io<+1>(smem, ld, fc, L, ZRepackIn{S, nzz, nzh, xa, has0, has1}, LineOut{});
            return;
        }
    }
    zrepack(S, smem + threadIdx.y * ld, nzz, nzh, has0, has1, xa);
    __syncthreads();
    dft_n<+1, FP>(smem, ld, fc, L);
}

// The L kz columns kz0 .. of the half spectra `in` into the shared lines (line
// c = column kz0 + c, zeros past nzh), a group of points' loads in flight at a time.
template <int U>
__device__ __forceinline__ void kzfill(float2* smem, const float2* __restrict__ in, int ld, int L, int lg, int kz0,
                                       int nxx, int nzh, int t0, int nthr) {
    batched_for<U>(
        t0, L * nxx, nthr,
        [&](int g) {
            const int c = g & (L - 1), ix = g >> lg;
            const int kz = kz0 + c;
            return (kz < nzh) ? in[(size_t)ix * nzh + kz] : make_float2(0.f, 0.f);
        },
        [&](int g, float2 v) { smem[(g & (L - 1)) * ld + (g >> lg)] = v; });
}

#define ZPASS_SETUP                                                  \
    extern __shared__ float2 smem[];                                 \
    __shared__ FFTPass s_pass[QP_MAXST];                             \
    const FFTCtx fc = make_ctx(a.pl, s_pass);                        \
    const int L = a.L, ld = a.pl.m, nzz = a.nzz, nxx = a.nxx;        \
    float2* line = smem + threadIdx.y * ld;                          \
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;             \
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;                 \
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;               \
    (void)r1;

// ---- z pass A ---------------------------------------------------------------
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) vz_passA_kernel(VzArgsA a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    __shared__ FFTPass s_pass_c[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const FFTCtx fcc = make_ctx(a.plc, s_pass_c);
    const int L = a.L, ld = max(a.pl.m, a.plc.m), nzz = a.nzz, nxx = a.nxx;
    float2* line = smem + threadIdx.y * ld;
    const int xa = blockIdx.x * 2 * L + 2 * threadIdx.y;
    const bool has0 = xa < nxx, has1 = xa + 1 < nxx;
    const size_t r0 = (size_t)xa * nzz, r1 = r0 + nzz;
    const int nzh = a.nzh;
    if (a.aux_spec) {
        zrepack_inverse<FP>(a.aux_spec, smem, ld, fc, L, nzz, nzh, has0, has1, xa);
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            const float2 v = line[k];
            if (has0) a.aux[r0 + k] = v.x;
            if (has1) a.aux[r1 + k] = v.y;
        }
        __syncthreads();
    }
    zload_pair(a.vz, line, nzz, has0, has1, r0, r1);
    __syncthreads();
    roundtrip_conv<FP>(smem, ld, fcc, L, a.HzM);
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
                r.pv.x = a.psi_vz[r0 + k];
                r.dx.x = a.Dx[r0 + k];
            }
            if (has1) {
                r.pv.y = a.psi_vz[r1 + k];
                r.dx.y = a.Dx[r1 + k];
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
    dft_n<-1, FP>(smem, ld, fc, L);
    zunpack(line, a.G, nzz, nzh, has0, has1, xa);
}

// ---- x-spectral pass ----------------------------------------------------------
// L kz columns per CTA (L a power of two); line c = column kz0 + c.
__device__ __forceinline__ float spec_symbol(const VxsArgs& a, int j, float k2) {
    if (a.mode == 0) {
        if (j == 1) return k2;
        const float k32 = exp2f(log2f(k2) * (1.f / 32.f));
        return (j == 0) ? k32 : k2 * k32;
    }
    const float ka = exp2f(0.505f * log2f(k2));
    if (a.mode == 1) return ka;
    const float num = 2.f * a.eta6 * ka * (1.f + a.tao * a.dt * ka);
    const float den = expf(-a.tao * a.tt * ka) + a.eta6 * expf(a.tao * a.dt * ka);
    return ka - num / den;
}

// FP: transform policy of the exact plan (Bluestein plans included).
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_PASS_REGS : QP_EXACT_REGS) vz_xspec_kernel(VxsArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.pl, s_pass);
    const int L = a.L, ld = a.pl.m, nxx = a.nxx, nzh = a.nzh;
    const int lg = 31 - __clz(L);
    const int kz0 = blockIdx.x * L;
    const int t0 = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    const int tot = L * nxx;
    const int nout = (a.mode == 0) ? 3 : 1;
    float2* X = smem + (size_t)L * ld;  // kept forward spectrum (three-output mode)
    float2* line = smem + threadIdx.y * ld;
    kzfill<x_epi_batch<FP>()>(smem, a.in, ld, L, lg, kz0, nxx, nzh, t0, nthr);
    __syncthreads();
    dft_n<-1, FP>(smem, ld, fc, L);
    if (nout == 3) {
        for (int ix = threadIdx.x; ix < nxx; ix += blockDim.x) X[threadIdx.y * ld + ix] = line[ix];
        __syncthreads();
    }
    // Outputs written out in sequence (a loop here costs register spills); the
    // indices are formed again inside each, so that none is held across the
    // transforms (this keeps the kernel within its register cap).
    auto output = [&](int j) __attribute__((always_inline)) {
        const int L = a.L, ld = a.pl.m, nzh = a.nzh, nxx = a.nxx;
        float2* out = (j == 0) ? a.out0 : (j == 1) ? a.out1 : a.out2;
        {
            const int kz = blockIdx.x * L + threadIdx.y;
            const float kzsq = a.kz2[(kz < nzh) ? kz : 0];
            float2* ln = smem + threadIdx.y * ld;
            const float2* src = (a.mode == 0) ? smem + (size_t)(L + threadIdx.y) * ld : ln;
            for (int ix = threadIdx.x; ix < nxx; ix += blockDim.x)
                ln[ix] = cscale(src[ix], spec_symbol(a, j, a.kx2[ix] + kzsq) * a.norm);
        }
        __syncthreads();
        dft_n<+1, FP>(smem, ld, fc, L);
        const int lgl = 31 - __clz(L), kzb = blockIdx.x * L, tl = L * nxx;
        for (int g = threadIdx.y * blockDim.x + threadIdx.x; g < tl; g += blockDim.x * blockDim.y) {
            const int c = g & (L - 1), ix = g >> lgl;
            if (kzb + c < nzh) out[(size_t)ix * nzh + kzb + c] = smem[c * ld + ix];
        }
        __syncthreads();
    };
    output(0);
    if (nout == 3) {
        output(1);
        output(2);
    }
}

// ---- x-spectral pass, stationary symbols as per-kz convolutions ---------------
// A stationary symbol s(kx, kz) acts on one kz column as a circular
// convolution along x, so a zero-padded FFT on the smooth convolution length
// replaces the exact (Bluestein) DFTs: one forward transform, then per output a
// multiply by the column's table and one inverse transform.
// NOUT = 3 (mode 0) or 1 (mode 1): each instance carries only the transforms it runs.
// FP: transform policy of the convolution plan.
template <int NOUT, class FP>
__global__ void __maxnreg__(NOUT == 3 ? QP_WIDE_REGS : FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS)
    vz_xspec_conv_kernel(VxsArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.plc, s_pass);
    const int L = a.L, m = a.plc.m, ld = m, nxx = a.nxx, nzh = a.nzh;
    const int lg = 31 - __clz(L);
    const int kz0 = blockIdx.x * L;
    const int t0 = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    const int tot = L * nxx;
    constexpr int nout = NOUT;
    float2* X = smem + (size_t)L * ld;  // kept forward spectrum (three-output mode)
    float2* line = smem + threadIdx.y * ld;
    kzfill<x_epi_batch<FP>()>(smem, a.in, ld, L, lg, kz0, nxx, nzh, t0, nthr);
    if constexpr (!FP::kCompiled)
        for (int k = nxx + threadIdx.x; k < m; k += blockDim.x) line[k] = make_float2(0.f, 0.f);
    __syncthreads();
    const int kz = min(kz0 + (int)threadIdx.y, nzh - 1);
    // the multipliers are even in k: rows hold entries 0..m/2
    const int mh = m / 2 + 1;
    if constexpr (FP::kCompiled) {
        // zero padding in the first pass; the last pass either keeps the
        // spectrum in X (three outputs) or applies the one multiplier
        if (nout == 3)
            FP::template run_io<-1>(smem, ld, fc, L, ZeroPadIn{nxx}, CopyOut{X + threadIdx.y * ld});
        else
            FP::template run_io<-1>(smem, ld, fc, L, ZeroPadIn{nxx}, EvenScaleOut{a.tab0 + (size_t)kz * mh, m});
    } else {
        fft_m<-1, FP>(smem, ld, fc, L);
        if (nout == 3) {
            for (int k = threadIdx.x; k < m; k += blockDim.x) X[threadIdx.y * ld + k] = line[k];
            __syncthreads();
        }
    }
    auto output = [&](const float* __restrict__ tab, float2* out) {
        const float2* src = (nout == 3) ? X + threadIdx.y * ld : line;
        const float* tk = tab + (size_t)kz * mh;
        if constexpr (FP::kCompiled) {
            // three outputs: the multiplier is applied as the first inverse pass loads X
            if (nout == 3) FP::template run_io<+1>(smem, ld, fc, L, EvenScaleIn{src, tk, m}, LineOut{});
            else FP::template run<+1>(smem, ld, fc, L);
        } else {
            for (int k = threadIdx.x; k < m; k += blockDim.x) line[k] = cscale(src[k], __ldg(&tk[min(k, m - k)]));
            __syncthreads();
            fft_m<+1, FP>(smem, ld, fc, L);
        }
        for (int g = t0; g < tot; g += nthr) {
            const int c = g & (L - 1), ix = g >> lg;
            if (kz0 + c < nzh) out[(size_t)ix * nzh + kz0 + c] = smem[c * ld + ix];
        }
        __syncthreads();
    };
    output(a.tab0, a.out0);
    if (nout == 3) {
        output(a.tab1, a.out1);
        output(a.tab2, a.out2);
    }
}

// One-time construction of the per-kz convolution multipliers (see VtabArgs).
// FP: transform policy of both plans (the run-time plan, or one compiled long
// plan when the exact length's Bluestein plan and the convolution plan are the
// same length, as the planner makes them for long lines).
template <class FP>
__global__ void __launch_bounds__(768, 1) vz_convtab_kernel(VtabArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    __shared__ FFTPass s_pass_c[QP_MAXST];
    const FFTCtx fe = make_ctx(a.pl, s_pass);
    const FFTCtx fcc = make_ctx(a.plc, s_pass_c);
    const int L = a.L, n = a.nxx, m = a.plc.m, ld = max(a.pl.m, a.plc.m);
    const int kz = blockIdx.x * L + threadIdx.y;
    const bool valid = kz < a.nzh;
    float2* line = smem + threadIdx.y * ld;
    const double kzsq = a.kz2[valid ? kz : 0];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double k2 = (double)a.kx2[k] + kzsq;
        double s;
        if (a.sym == 4) s = a.V[(size_t)((k < a.nxh) ? k : n - k) * a.nzh + (valid ? kz : 0)];
        else if (a.sym == 1) s = k2;
        else if (a.sym == 0) s = pow(k2, 1.0 / 32.0);
        else if (a.sym == 2) s = pow(k2, 33.0 / 32.0);
        else s = pow(k2, 0.505);
        line[k] = make_float2((float)s, 0.f);
    }
    __syncthreads();
    dft_n<+1, FP>(smem, ld, fe, L);  // sum_k s e^{+2 pi i k d/n}
    // wrap to length m: lags 0..n-1 stay, lags -(n-1)..-1 go to m-n+1..m-1 (m >= 2n-1)
    if (m > n) {
        for (int dd = 1 + threadIdx.x; dd < n; dd += blockDim.x) line[m - dd] = line[n - dd];
        __syncthreads();
        for (int k = n + threadIdx.x; k <= m - n; k += blockDim.x) line[k] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) line[k] = make_float2(line[k].x * a.norm, 0.f);
    __syncthreads();
    fft_m<-1, FP>(smem, ld, fcc, L);
    // the wrapped kernel is even, so its transform is real and even: keep 0..m/2
    const int mh = m / 2 + 1;
    if (valid)
        for (int k = threadIdx.x; k < mh; k += blockDim.x) a.out[(size_t)kz * mh + k] = line[k].x / (float)m;
}

// ---- z pass B -----------------------------------------------------------------
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) vz_passB_kernel(VzArgsB a) {
    ZPASS_SETUP
    const int nzh = a.nzh;
    float2* acc = smem + (size_t)(L + threadIdx.y) * ld;  // running total of this line pair
    // three terms, written out in sequence (a loop here costs register spills)
    auto term = [&](const float2* spec, const float* cf, float sg, bool first) {
        zrepack_inverse<FP>(spec, smem, ld, fc, L, nzz, nzh, has0, has1, xa);
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            const float2 y = line[k];
            float2 t = first ? make_float2(0.f, 0.f) : acc[k];
            if (has0) t.x += sg * cf[r0 + k] * y.x;
            if (has1) t.y += sg * cf[r1 + k] * y.y;
            acc[k] = t;
        }
        __syncthreads();
    };
    term(a.Y2, a.y2, 1.f, true);
    term(a.Y3, a.y3c, -1.f, false);
    term(a.Y4, a.y4c, -1.f, false);
    struct TIn {
        float2 y1, dv;
    };
    batched_for<kEpiBatchZ>(
        threadIdx.x, nzz, blockDim.x,
        [&](int k) {
            TIn r{};
            if (has0) {
                r.y1.x = a.y1[r0 + k];
                r.dv.x = a.div[r0 + k];
            }
            if (has1) {
                r.y1.y = a.y1[r1 + k];
                r.dv.y = a.div[r1 + k];
            }
            return r;
        },
        [&](int k, const TIn& r) {
            const float2 t = acc[k];
            float2 v = make_float2(0.f, 0.f);
            if (has0) {
                v.x = r.y1.x * r.dv.x + t.x;
                a.total[r0 + k] = v.x;
            }
            if (has1) {
                v.y = r.y1.y * r.dv.y + t.y;
                a.total[r1 + k] = v.y;
            }
            line[k] = v;
        });
    __syncthreads();
    dft_n<-1, FP>(smem, ld, fc, L);
    zunpack(line, a.T, nzz, nzh, has0, has1, xa);
}

// ---- z pass C -----------------------------------------------------------------
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) vz_passC_kernel(VzArgsC a) {
    ZPASS_SETUP
    const int nzh = a.nzh;
    if (a.Dspec) {
        zrepack_inverse<FP>(a.Dspec, smem, ld, fc, L, nzz, nzh, has0, has1, xa);
    }
    struct PIn {
        float2 p, e1, tot, e2, e3, aux;
    };
    batched_for<kEpiBatchZ>(
        threadIdx.x, nzz, blockDim.x,
        [&](int k) {
            PIn r{};
            if (has0) {
                const size_t i = r0 + k;
                r.p.x = a.p[i];
                r.e1.x = a.e1[i];
                r.tot.x = a.total[i];
                r.e2.x = a.e2[i];
                r.e3.x = a.e3[i];
                r.aux.x = a.aux[i];
            }
            if (has1) {
                const size_t i = r1 + k;
                r.p.y = a.p[i];
                r.e1.y = a.e1[i];
                r.tot.y = a.total[i];
                r.e2.y = a.e2[i];
                r.e3.y = a.e3[i];
                r.aux.y = a.aux[i];
            }
            return r;
        },
        [&](int k, const PIn& r) {
            const float2 D = a.Dspec ? line[k] : make_float2(0.f, 0.f);
            float2 pn = make_float2(0.f, 0.f);
            if (has0) {
                pn.x = r.p.x + r.e1.x * (r.tot.x + a.sgn * r.e2.x * D.x) + a.sgn * r.e3.x * r.aux.x;
                if (xa == a.xs && k == a.zs) pn.x += a.src;
            }
            if (has1) {
                pn.y = r.p.y + r.e1.y * (r.tot.y + a.sgn * r.e2.y * D.y) + a.sgn * r.e3.y * r.aux.y;
                if (xa + 1 == a.xs && k == a.zs) pn.y += a.src;
            }
            line[k] = pn;
        });
    __syncthreads();
    const int ix0 = blockIdx.x * 2 * L;
    if (a.rec_off) {
        float* sf = reinterpret_cast<float*>(smem);
        const int t0 = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
        const int q0 = a.rec_off[blockIdx.x], q1 = a.rec_off[blockIdx.x + 1];
        for (int q = q0 + t0; q < q1; q += nthr) {
            const RecEntry e = a.rec[q];
            const int rel = e.gx - ix0;
            const int si = 2 * ((rel >> 1) * ld + e.gz) + (rel & 1);
            if (a.gather_row) a.gather_row[e.ir] = sf[si];
            if (a.obs_row && e.inject) sf[si] = a.obs_row[e.ir];
        }
        __syncthreads();
    }
    const int pml = a.pml, nz = nzz - 2 * pml;
    if (!a.ssg && !a.img) {
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            const float2 pn = line[k];
            if (has0) a.p[r0 + k] = pn.x;
            if (has1) a.p[r1 + k] = pn.y;
        }
    } else {
        // sums of the interior (illumination, image) and the source
        // wavefield of both rows, loaded a group of points at a time
        struct Acc {
            float s[2], sc[2], m[2], mc[2], ps[2];
        };
        batched_for<kEpiBatchZ>(
            threadIdx.x, nzz, blockDim.x,
            [&](int k) {
                Acc r{};
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int ix = xa + h;
                    if (ix < nxx && ix >= pml && ix < nxx - pml && k >= pml && k < nzz - pml) {
                        const size_t j = (size_t)(ix - pml) * nz + (k - pml);
                        if (a.ssg) {
                            r.s[h] = a.ssg[j];
                            r.sc[h] = a.ssg_c[j];
                        }
                        if (a.img) {
                            r.m[h] = a.img[j];
                            r.mc[h] = a.img_c[j];
                            r.ps[h] = a.ps[(size_t)ix * nzz + k];
                        }
                    }
                }
                return r;
            },
            [&](int k, const Acc& r) {
                const float2 pn = line[k];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int ix = xa + h;
                    if (ix >= nxx) break;
                    const float v = h ? pn.y : pn.x;
                    a.p[(size_t)ix * nzz + k] = v;
                    if (ix >= pml && ix < nxx - pml && k >= pml && k < nzz - pml) {
                        const size_t j = (size_t)(ix - pml) * nz + (k - pml);
                        if (a.ssg) kahan_add_v(a.ssg, a.ssg_c, j, r.s[h], r.sc[h], v * v);
                        if (a.img) kahan_add_v(a.img, a.img_c, j, r.m[h], r.mc[h], r.ps[h] * v);
                    }
                }
            });
    }
    __syncthreads();
    // forward z transform of the new p: half spectrum for the aux operator and
    // the staggered z derivative from the same transform
    dft_n<-1, FP>(smem, ld, fc, L);
    zunpack(line, a.P, nzz, nzh, has0, has1, xa);
    __syncthreads();
    if constexpr (FP::kCompiled) {
        if (!fc.blue) {
            // the multiplier applied as the first inverse pass loads the line
            FP::template run_io<+1>(smem, ld, fc, L, MulIn{a.HzP}, LineOut{});
        } else {
            for (int k = threadIdx.x; k < nzz; k += blockDim.x) line[k] = cmul(line[k], __ldg(&a.HzP[k]));
            __syncthreads();
            dft_n<+1, FP>(smem, ld, fc, L);
        }
    } else {
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) line[k] = cmul(line[k], __ldg(&a.HzP[k]));
        __syncthreads();
        dft_n<+1, FP>(smem, ld, fc, L);
    }
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
                r.pp.x = a.psi_pz[r0 + k];
                r.v0.x = a.vz[r0 + k];
                r.bb.x = a.bbz[r0 + k];
            }
            if (has1) {
                r.pp.y = a.psi_pz[r1 + k];
                r.v0.y = a.vz[r1 + k];
                r.bb.y = a.bbz[r1 + k];
            }
            return r;
        },
        [&](int k, const VIn& r) {
            const float2 d = line[k];
            if (has0) {
                const float ps = r.hb * r.pp.x + r.ha * d.x;
                a.psi_pz[r0 + k] = ps;
                a.vz[r0 + k] = r.v0.x + a.dt * r.bb.x * (d.x + ps);
            }
            if (has1) {
                const float ps = r.hb * r.pp.y + r.ha * d.y;
                a.psi_pz[r1 + k] = ps;
                a.vz[r1 + k] = r.v0.y + a.dt * r.bb.y * (d.y + ps);
            }
        });
}

// ---- z inverse only -------------------------------------------------------------
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) vz_zinv_kernel(VzArgsI a) {
    ZPASS_SETUP
    zrepack_inverse<FP>(a.spec, smem, ld, fc, L, nzz, a.nzh, has0, has1, xa);
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 v = line[k];
        if (has0) a.out[r0 + k] = v.x;
        if (has1) a.out[r1 + k] = v.y;
    }
}

// ---- low-rank form ------------------------------------------------------------------
// x-spectral pass of the low-rank pressure term: one forward transform of the
// kz column of G, then per factor b a multiply by its per-kz convolution table
// and an inverse transform (the factor loop keeps one copy of the inverse code).
template <class FP>
__global__ void __maxnreg__(QP_WIDE_REGS) lr_xconv_kernel(LrxArgs a) {
    extern __shared__ float2 smem[];
    __shared__ FFTPass s_pass[QP_MAXST];
    const FFTCtx fc = make_ctx(a.plc, s_pass);
    const int L = a.L, m = a.plc.m, ld = m, nxx = a.nxx, nzh = a.nzh;
    const int lg = 31 - __clz(L);
    const int kz0 = blockIdx.x * L;
    const int t0 = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    const int tot = L * nxx;
    float2* X = smem + (size_t)L * ld;  // kept forward spectrum
    float2* line = smem + threadIdx.y * ld;
    kzfill<x_epi_batch<FP>()>(smem, a.in, ld, L, lg, kz0, nxx, nzh, t0, nthr);
    if constexpr (FP::kCompiled) {
        // zero padding in the first pass, the spectrum straight into X
        __syncthreads();
        FP::template run_io<-1>(smem, ld, fc, L, ZeroPadIn{nxx}, CopyOut{X + threadIdx.y * ld});
    } else {
        for (int k = nxx + threadIdx.x; k < m; k += blockDim.x) line[k] = make_float2(0.f, 0.f);
        __syncthreads();
        fft_m<-1, FP>(smem, ld, fc, L);
        for (int k = threadIdx.x; k < m; k += blockDim.x) X[threadIdx.y * ld + k] = line[k];
    }
    const int kz = min(kz0 + (int)threadIdx.y, nzh - 1);
    const int mh = m / 2 + 1;
#pragma unroll 1
    for (int b = 0; b < a.row; b++) {
        const float* tk = a.tab + ((size_t)b * nzh + kz) * mh;
        __syncthreads();
        if constexpr (FP::kCompiled) {
            // the multiplier applied as the first inverse pass loads X
            FP::template run_io<+1>(smem, ld, fc, L, EvenScaleIn{X + threadIdx.y * ld, tk, m}, LineOut{});
        } else {
            for (int k = threadIdx.x; k < m; k += blockDim.x)
                line[k] = cscale(X[threadIdx.y * ld + k], __ldg(&tk[min(k, m - k)]));
            __syncthreads();
            fft_m<+1, FP>(smem, ld, fc, L);
        }
        float2* out = a.out + (size_t)b * nxx * nzh;
        for (int g = t0; g < tot; g += nthr) {
            const int c = g & (L - 1), ix = g >> lg;
            if (kz0 + c < nzh) out[(size_t)ix * nzh + kz0 + c] = smem[c * ld + ix];
        }
    }
}

// z pass of the low-rank pressure term: psc (+)= sum_b c_b(x) q_b(x) over the
// factors b0 .. b0+nb-1 (nb <= lr_terms<FP>()), q_b the inverse z transform of
// half spectrum b; the first launch (b0 = 0) overwrites psc.  The factors are
// written out in sequence like z pass B's terms: a loop around the transform
// spills registers.  The run-time-plan instances take one factor per launch
// (three copies of their radix switch spilled 3 KB).
template <class FP> constexpr int lr_terms() { return FP::kCompiled ? 3 : 1; }
template <class FP>
__global__ void __maxnreg__(FP::kMaxRadix <= 12 ? QP_R12_REGS : QP_PASS_REGS) lr_zsum_kernel(LrsArgs a, int b0, int nb) {
    ZPASS_SETUP
    const int nzh = a.nzh;
    float2* acc = smem + (size_t)(L + threadIdx.y) * ld;
    auto term = [&](int b, bool first) {
        zrepack_inverse<FP>(a.Q + (size_t)b * nxx * nzh, smem, ld, fc, L, nzz, nzh, has0, has1, xa);
        const float* cb = a.c + (size_t)b * nxx * nzz;
        for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
            const float2 v = line[k];
            float2 t = first ? make_float2(0.f, 0.f) : acc[k];
            if (has0) t.x = fmaf(__ldg(&cb[r0 + k]), v.x, t.x);
            if (has1) t.y = fmaf(__ldg(&cb[r1 + k]), v.y, t.y);
            acc[k] = t;
        }
        __syncthreads();
    };
    term(b0, true);
    if (lr_terms<FP>() > 1 && nb > 1) term(b0 + 1, false);
    if (lr_terms<FP>() > 2 && nb > 2) term(b0 + 2, false);
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const float2 t = acc[k];
        if (has0) a.psc[r0 + k] = b0 ? a.psc[r0 + k] + t.x : t.x;
        if (has1) a.psc[r1 + k] = b0 ? a.psc[r1 + k] + t.y : t.y;
    }
}

}  // namespace qp
