// fftline.cuh -- shared-memory line FFT engine for the PSTD step kernels.
//
// A CTA holds a tile of L complex lines in shared memory (line stride `ld`
// float2).  Two real field lines are packed into one complex line (re = line
// a, im = line b); every spectral operator applied here has a Hermitian
// symbol, so the packed transform returns the two real results in re/im.
//
// Transforms are Stockham autosort, mixed radix {2,3,4,5,7,11,13}, ping-pong
// between two shared buffers.  A length whose factorisation holds a larger
// prime (439, 2461 = 23*107, 860 = 4*5*43 ...) goes through Bluestein's
// chirp-z identity with a {2,3,5,7}-smooth inner length m >= 2n-1, so the
// k-grid is exactly the reference's (cufftPlan2d on the unpadded window,
// sgpstd-qmodeling/acps4.cu:871).
#pragma once
#include <cuda_runtime.h>

#include "qpstd_internal.h"

namespace qp {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by (sgn * i)
__device__ __forceinline__ float2 cmuli(float2 a, float sgn) { return make_float2(-sgn * a.y, sgn * a.x); }

// cos / sin of 2*pi*m/P (mathematical constants)
template <int P> struct Tw;
template <> struct Tw<3> {
    __device__ __forceinline__ static float c(int m) {
        constexpr float t[3] = {1.f, -0.5f, -0.5f};
        return t[m];
    }
    __device__ __forceinline__ static float s(int m) {
        constexpr float t[3] = {0.f, 0.86602540378443871f, -0.86602540378443871f};
        return t[m];
    }
};
template <> struct Tw<5> {
    __device__ __forceinline__ static float c(int m) {
        constexpr float t[5] = {1.f, 0.30901699437494745f, -0.80901699437494734f, -0.80901699437494734f,
                                   0.30901699437494745f};
        return t[m];
    }
    __device__ __forceinline__ static float s(int m) {
        constexpr float t[5] = {0.f, 0.95105651629515353f, 0.58778525229247325f, -0.58778525229247325f,
                                   -0.95105651629515353f};
        return t[m];
    }
};
template <> struct Tw<7> {
    __device__ __forceinline__ static float c(int m) {
        constexpr float t[7] = {1.f, 0.62348980185873359f, -0.22252093395631434f, -0.90096886790241903f,
                                   -0.90096886790241903f, -0.22252093395631434f, 0.62348980185873359f};
        return t[m];
    }
    __device__ __forceinline__ static float s(int m) {
        constexpr float t[7] = {0.f, 0.7818314824680298f, 0.97492791218182362f, 0.43388373911755823f,
                                   -0.43388373911755823f, -0.97492791218182362f, -0.7818314824680298f};
        return t[m];
    }
};
template <> struct Tw<11> {
    __device__ __forceinline__ static float c(int m) {
        constexpr float t[11] = {1.f, 0.84125353283118121f, 0.41541501300188644f, -0.142314838273285f,
                                    -0.65486073394528499f, -0.95949297361449737f, -0.95949297361449737f,
                                    -0.65486073394528499f, -0.142314838273285f, 0.41541501300188644f,
                                    0.84125353283118121f};
        return t[m];
    }
    __device__ __forceinline__ static float s(int m) {
        constexpr float t[11] = {0.f, 0.54064081745559756f, 0.90963199535451833f, 0.9898214418809328f,
                                    0.75574957435425827f, 0.28173255684142967f, -0.28173255684142967f,
                                    -0.75574957435425827f, -0.9898214418809328f, -0.90963199535451833f,
                                    -0.54064081745559756f};
        return t[m];
    }
};
template <> struct Tw<13> {
    __device__ __forceinline__ static float c(int m) {
        constexpr float t[13] = {1.f, 0.88545602565320991f, 0.56806474673115592f, 0.12053668025532301f,
                                    -0.35460488704253545f, -0.74851074817110119f, -0.97094181742605201f,
                                    -0.97094181742605201f, -0.74851074817110119f, -0.35460488704253545f,
                                    0.12053668025532301f, 0.56806474673115592f, 0.88545602565320991f};
        return t[m];
    }
    __device__ __forceinline__ static float s(int m) {
        constexpr float t[13] = {0.f, 0.46472317204376851f, 0.82298386589365635f, 0.99270887409805397f,
                                    0.93501624268541483f, 0.66312265824079519f, 0.23931566428755768f,
                                    -0.23931566428755768f, -0.66312265824079519f, -0.93501624268541483f,
                                    -0.99270887409805397f, -0.82298386589365635f, -0.46472317204376851f};
        return t[m];
    }
};

// In-register DFT of size P; sgn = -1 forward (e^{-i}), +1 inverse.
template <int P> __device__ __forceinline__ void dftP(float2 (&v)[P], float sgn);

template <> __device__ __forceinline__ void dftP<2>(float2 (&v)[2], float) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <> __device__ __forceinline__ void dftP<4>(float2 (&v)[4], float sgn) {
    float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    float2 t2 = cadd(v[1], v[3]), t3 = cmuli(csub(v[1], v[3]), sgn);
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
}

// odd P: X_q = v0 + sum_r (v_r + v_{P-r}) cos(2 pi r q/P) + sgn i (v_r - v_{P-r}) sin(2 pi r q/P)
template <int P> __device__ __forceinline__ void dft_odd(float2 (&v)[P], float sgn) {
    constexpr int H = (P - 1) / 2;
    float2 a[H], b[H];
#pragma unroll
    for (int r = 1; r <= H; r++) {
        a[r - 1] = cadd(v[r], v[P - r]);
        b[r - 1] = csub(v[r], v[P - r]);
    }
    float2 x0 = v[0];
    float2 s0 = x0;
#pragma unroll
    for (int r = 0; r < H; r++) s0 = cadd(s0, a[r]);
#pragma unroll
    for (int q = 1; q <= H; q++) {
        float2 re = x0, im = make_float2(0.f, 0.f);
#pragma unroll
        for (int r = 1; r <= H; r++) {
            const int m = (r * q) % P;
            re.x = fmaf(a[r - 1].x, Tw<P>::c(m), re.x);
            re.y = fmaf(a[r - 1].y, Tw<P>::c(m), re.y);
            im.x = fmaf(b[r - 1].x, Tw<P>::s(m), im.x);
            im.y = fmaf(b[r - 1].y, Tw<P>::s(m), im.y);
        }
        float2 ii = cmuli(im, sgn);
        v[q] = cadd(re, ii);
        v[P - q] = csub(re, ii);
    }
    v[0] = s0;
}
template <> __device__ __forceinline__ void dftP<3>(float2 (&v)[3], float sgn) { dft_odd<3>(v, sgn); }
template <> __device__ __forceinline__ void dftP<5>(float2 (&v)[5], float sgn) { dft_odd<5>(v, sgn); }
template <> __device__ __forceinline__ void dftP<7>(float2 (&v)[7], float sgn) { dft_odd<7>(v, sgn); }
template <> __device__ __forceinline__ void dftP<11>(float2 (&v)[11], float sgn) { dft_odd<11>(v, sgn); }
template <> __device__ __forceinline__ void dftP<13>(float2 (&v)[13], float sgn) { dft_odd<13>(v, sgn); }

// One Stockham stage over L lines of length m (stride ld): src -> dst.
template <int P>
__device__ __forceinline__ void fft_stage(const float2* __restrict__ src, float2* __restrict__ dst, int L, int ld,
                                          int m, int ns, const float2* __restrict__ w, float sgn) {
    const int nbl = m / P;
    const int total = L * nbl;
    const int tstride = m / (ns * P);
    for (int g = threadIdx.x; g < total; g += blockDim.x) {
        const int l = g / nbl;
        const int j = g - l * nbl;
        const int k = j % ns;
        const float2* s = src + l * ld;
        float2 v[P];
        v[0] = s[j];
#pragma unroll
        for (int r = 1; r < P; r++) {
            float2 t = __ldg(&w[r * k * tstride]);
            t.y *= -sgn;  // w holds e^{-2 pi i k/m}; sgn=-1 keeps it, +1 conjugates
            v[r] = cmul(s[j + r * nbl], t);
        }
        dftP<P>(v, sgn);
        float2* d = dst + l * ld;
        const int base = (j - k) * P + k;
#pragma unroll
        for (int r = 0; r < P; r++) d[base + r * ns] = v[r];
    }
}

// Full length-m transform of the L lines in `a`; returns the buffer holding
// the result (a or b).  Ends with __syncthreads().
__device__ __forceinline__ float2* fft_core(float2* a, float2* b, int L, int ld, const FFTPlanDev& pl, float sgn) {
    int ns = 1;
    for (int s = 0; s < pl.nst; s++) {
        const int P = pl.rad[s];
        switch (P) {
            case 2: fft_stage<2>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            case 3: fft_stage<3>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            case 4: fft_stage<4>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            case 5: fft_stage<5>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            case 7: fft_stage<7>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            case 11: fft_stage<11>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
            default: fft_stage<13>(a, b, L, ld, pl.m, ns, pl.w, sgn); break;
        }
        __syncthreads();
        float2* t = a;
        a = b;
        b = t;
        ns *= P;
    }
    return a;
}

// Exact length-n DFT of the L lines in `a` (entries [0,n) of each line).
// sgn = -1 forward, +1 inverse (unnormalised).  Result in entries [0,n) of the
// returned buffer.  Caller must have synchronised after filling `a`.
__device__ __forceinline__ float2* dft_lines(float2* a, float2* b, int L, int ld, const FFTPlanDev& pl, float sgn) {
    if (!pl.blue) return fft_core(a, b, L, ld, pl, sgn);
    const int n = pl.n, m = pl.m;
    const float cs = (sgn > 0.f) ? -1.f : 1.f;  // inverse: DFT of the conjugate, conjugated
    for (int g = threadIdx.x; g < L * m; g += blockDim.x) {
        const int l = g / m, k = g - l * m;
        float2 v = make_float2(0.f, 0.f);
        if (k < n) {
            float2 x = a[l * ld + k];
            x.y *= cs;
            v = cmul(x, __ldg(&pl.chirp[k]));
        }
        a[l * ld + k] = v;
    }
    __syncthreads();
    float2* r = fft_core(a, b, L, ld, pl, -1.f);
    float2* o = (r == a) ? b : a;
    for (int g = threadIdx.x; g < L * m; g += blockDim.x) {
        const int l = g / m, k = g - l * m;
        r[l * ld + k] = cmul(r[l * ld + k], __ldg(&pl.bhat[k]));
    }
    __syncthreads();
    r = fft_core(r, o, L, ld, pl, +1.f);
    for (int g = threadIdx.x; g < L * n; g += blockDim.x) {
        const int l = g / n, k = g - l * n;
        float2 y = cmul(r[l * ld + k], __ldg(&pl.chirp[k]));
        y.y *= cs;
        r[l * ld + k] = y;
    }
    __syncthreads();
    return r;
}

// y = IDFT( H .* DFT(x) ) on L packed lines; H is a complex table of length n
// (already divided by n).  Returns the buffer with the result.
__device__ __forceinline__ float2* roundtrip_c(float2* a, float2* b, int L, int ld, const FFTPlanDev& pl,
                                               const float2* __restrict__ H) {
    float2* r = dft_lines(a, b, L, ld, pl, -1.f);
    const int n = pl.n;
    for (int g = threadIdx.x; g < L * n; g += blockDim.x) {
        const int l = g / n, k = g - l * n;
        r[l * ld + k] = cmul(r[l * ld + k], __ldg(&H[k]));
    }
    __syncthreads();
    float2* o = (r == a) ? b : a;
    return dft_lines(r, o, L, ld, pl, +1.f);
}

// Same with a real symbol.
__device__ __forceinline__ float2* roundtrip_r(float2* a, float2* b, int L, int ld, const FFTPlanDev& pl,
                                               const float* __restrict__ H) {
    float2* r = dft_lines(a, b, L, ld, pl, -1.f);
    const int n = pl.n;
    for (int g = threadIdx.x; g < L * n; g += blockDim.x) {
        const int l = g / n, k = g - l * n;
        r[l * ld + k] = cscale(r[l * ld + k], __ldg(&H[k]));
    }
    __syncthreads();
    float2* o = (r == a) ? b : a;
    return dft_lines(r, o, L, ld, pl, +1.f);
}

}  // namespace qp
