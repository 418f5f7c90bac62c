// fft_reg.cuh -- register-blocked line FFT for the PSTD pass kernels.
//
// A CTA of TX x L threads holds L complex lines (stride ld float2) in shared
// memory; thread (x, y) works on line y.  A length-m transform is a sequence
// of Stockham passes of radix R <= 16; in a pass every active thread loads the
// R inputs of one butterfly into registers, applies the twiddles, runs an
// in-register DFT of size R (nested Cooley-Tukey with compile-time roots of
// unity), and after a barrier stores the R outputs in place.  TX is chosen so
// that one butterfly per thread covers the line (TX >= m / min R).
//
// Lengths with a prime factor above 13 use Bluestein's identity with a
// {2,3,5,7}-smooth inner length m >= 2n-1 (the k-grid stays the reference's,
// cufftPlan2d on the window, sgpstd-qmodeling/acps4.cu:871).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qpstd_internal.h"

namespace qp {

// ---- complex helpers ----------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// ---- compile-time roots of unity (Taylor series, evaluated by the compiler) ----
constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr double ct_cos(double x) {
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 40; i++) {
        term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
        sum += term;
    }
    return sum;
}
constexpr double ct_sin(double x) {
    double term = x, sum = x;
    for (int i = 1; i < 40; i++) {
        term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
        sum += term;
    }
    return sum;
}
// c[m] + i s[m] = exp(2 pi i m / R)
template <int R> struct Roots {
    float c[R];
    float s[R];
    constexpr Roots() : c(), s() {
        for (int m = 0; m < R; m++) {
            double a = 2.0 * kPiD * m / R;
            if (a > kPiD) a -= 2.0 * kPiD;
            c[m] = (float)ct_cos(a);
            s[m] = (float)ct_sin(a);
        }
    }
};

template <int R> constexpr int small_factor() {
    for (int f = 2; f * f <= R; f++)
        if (R % f == 0) return f;
    return R;
}

// ---- in-register DFTs, S = -1 forward (e^{-i}), +1 inverse ---------------------
template <int R, int S> __device__ __forceinline__ void dft(float2 (&v)[R]);

template <int P, int S> __device__ __forceinline__ void dft_prime(float2 (&v)[P]) {
    if constexpr (P == 2) {
        const float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else {
        constexpr int H = (P - 1) / 2;
        constexpr Roots<P> rt{};
        float2 a[H], b[H];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            a[r - 1] = cadd(v[r], v[P - r]);
            b[r - 1] = csub(v[r], v[P - r]);
        }
        const float2 x0 = v[0];
        float2 s0 = x0;
#pragma unroll
        for (int r = 0; r < H; r++) s0 = cadd(s0, a[r]);
#pragma unroll
        for (int q = 1; q <= H; q++) {
            float2 re = x0, im = make_float2(0.f, 0.f);
#pragma unroll
            for (int r = 1; r <= H; r++) {
                const int m = (r * q) % P;
                re.x = fmaf(a[r - 1].x, rt.c[m], re.x);
                re.y = fmaf(a[r - 1].y, rt.c[m], re.y);
                im.x = fmaf(b[r - 1].x, rt.s[m], im.x);
                im.y = fmaf(b[r - 1].y, rt.s[m], im.y);
            }
            // + S i im
            const float2 ii = make_float2(-(float)S * im.y, (float)S * im.x);
            v[q] = cadd(re, ii);
            v[P - q] = csub(re, ii);
        }
        v[0] = s0;
    }
}

template <int R, int S> __device__ __forceinline__ void dft(float2 (&v)[R]) {
    if constexpr (R == 1) {
        return;
    } else if constexpr (R == 4) {
        const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        const float2 d = csub(v[1], v[3]);
        const float2 t2 = cadd(v[1], v[3]);
        const float2 t3 = make_float2(-(float)S * d.y, (float)S * d.x);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else if constexpr (small_factor<R>() == R) {
        dft_prime<R, S>(v);
    } else {
        // R = A * B, A the smallest factor (R = 8, 16 split as 4 * ...)
        constexpr int A0 = small_factor<R>();
        constexpr int A = (A0 == 2 && R % 4 == 0 && R > 4) ? 4 : A0;
        constexpr int B = R / A;
        constexpr Roots<R> rt{};
        float2 u[A][B];
#pragma unroll
        for (int a = 0; a < A; a++) {
#pragma unroll
            for (int b = 0; b < B; b++) u[a][b] = v[a + A * b];
            dft<B, S>(u[a]);
        }
#pragma unroll
        for (int a = 1; a < A; a++)
#pragma unroll
            for (int q = 1; q < B; q++) {
                const int m = (a * q) % R;
                u[a][q] = cmul(u[a][q], make_float2(rt.c[m], (float)S * rt.s[m]));
            }
#pragma unroll
        for (int q = 0; q < B; q++) {
            float2 t[A];
#pragma unroll
            for (int a = 0; a < A; a++) t[a] = u[a][q];
            dft<A, S>(t);
#pragma unroll
            for (int p = 0; p < A; p++) v[q + B * p] = t[p];
        }
    }
}

// ---- one Stockham pass over the lines of the CTA (in place) ------------------------
// Thread (threadIdx.x, threadIdx.y) handles butterfly j = threadIdx.x of line
// threadIdx.y.  The radix is a runtime value; all radices share one RMAX-entry
// register array (constant indices under full unrolling), so one copy of the
// pass serves every plan without register spills.  RMAX is 16, or 12 for
// kernels whose plans use radices up to 12 only (the array then takes 8
// registers fewer, which lets those kernels run under a lower register cap).
// Ends with a barrier.
template <int R, int N> __device__ __forceinline__ float2 (&head(float2 (&v)[N]))[R] {
    return *reinterpret_cast<float2(*)[R]>(&v[0]);
}

template <int S, int RMAX = 16>
__device__ __forceinline__ void reg_pass(float2* buf, int ld, const FFTPass& ps, const float2* __restrict__ tw,
                                         int L) {
    static_assert(RMAX == 12 || RMAX == 16, "register array of 12 or 16 entries");
    const int R = ps.R;
    const int j = threadIdx.x;
    const int l = threadIdx.y;
    const bool act = (j < ps.B) && (l < L);
    float2 v[RMAX];
    int k = 0;
    float2* line = buf + l * ld;
    if (act) {
        k = (ps.ns == 1) ? 0 : (int)(j - __umulhi((unsigned)j, ps.ns_magic) * ps.ns);
#pragma unroll
        for (int r = 0; r < RMAX; r++)
            if (r < R) v[r] = line[j + r * ps.B];
        if (ps.ns > 1) {
            float2 w1 = __ldg(&tw[k * ps.twstride]);
            if (S > 0) w1.y = -w1.y;
            float2 w = w1;
#pragma unroll
            for (int r = 1; r < RMAX; r++)
                if (r < R) {
                    v[r] = cmul(v[r], w);
                    w = cmul(w, w1);
                }
        }
        if constexpr (RMAX == 16) {
            switch (R) {
                case 2: dft<2, S>(head<2>(v)); break;
                case 3: dft<3, S>(head<3>(v)); break;
                case 4: dft<4, S>(head<4>(v)); break;
                case 5: dft<5, S>(head<5>(v)); break;
                case 6: dft<6, S>(head<6>(v)); break;
                case 7: dft<7, S>(head<7>(v)); break;
                case 8: dft<8, S>(head<8>(v)); break;
                case 9: dft<9, S>(head<9>(v)); break;
                case 10: dft<10, S>(head<10>(v)); break;
                case 11: dft<11, S>(head<11>(v)); break;
                case 12: dft<12, S>(head<12>(v)); break;
                case 13: dft<13, S>(head<13>(v)); break;
                case 14: dft<14, S>(head<14>(v)); break;
                case 15: dft<15, S>(head<15>(v)); break;
                default: dft<16, S>(head<16>(v)); break;
            }
        } else {
            switch (R) {
                case 2: dft<2, S>(head<2>(v)); break;
                case 3: dft<3, S>(head<3>(v)); break;
                case 4: dft<4, S>(head<4>(v)); break;
                case 5: dft<5, S>(head<5>(v)); break;
                case 6: dft<6, S>(head<6>(v)); break;
                case 7: dft<7, S>(head<7>(v)); break;
                case 8: dft<8, S>(head<8>(v)); break;
                case 9: dft<9, S>(head<9>(v)); break;
                case 10: dft<10, S>(head<10>(v)); break;
                case 11: dft<11, S>(head<11>(v)); break;
                default: dft<12, S>(head<12>(v)); break;
            }
        }
    }
    __syncthreads();
    if (act) {
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < RMAX; r++)
            if (r < R) line[base + r * ps.ns] = v[r];
    }
    __syncthreads();
}

// Length-m transform (unnormalised) of the L lines, in place.
template <int S, int RMAX = 16>
__device__ __forceinline__ void fft_m_impl(float2* buf, int ld, const FFTPass* __restrict__ sp, int nst,
                                           const float2* __restrict__ tw, int L) {
    for (int i = 0; i < nst; i++) {
        const FFTPass ps = sp[i];
        reg_pass<S, RMAX>(buf, ld, ps, tw, L);
    }
}

// The plan as the kernels use it: scalars in registers, passes in shared memory.
struct FFTCtx {
    int n, m, blue, nst;
    const FFTPass* sp;
    const float2 *w, *chirp, *bhat;
};

// Copies the plan's passes to shared memory (constant indices, so the plan
// stays in the parameter bank); ends with a barrier.
__device__ __forceinline__ FFTCtx make_ctx(const FFTPlanDev& pl, FFTPass* s_pass) {
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
#pragma unroll
    for (int i = 0; i < QP_MAXST; i++)
        if (t == i && i < pl.nst) s_pass[i] = pl.pass[i];
    __syncthreads();
    FFTCtx c;
    c.n = pl.n;
    c.m = pl.m;
    c.blue = pl.blue;
    c.nst = pl.nst;
    c.sp = s_pass;
    c.w = pl.w;
    c.chirp = pl.chirp;
    c.bhat = pl.bhat;
    return c;
}

// ---- transform policies ---------------------------------------------------------
// A pass kernel is compiled for one policy, the way it runs its length-m
// transforms:
//   RtFFT<RMAX>  the plan's radices read at run time (any plan the host builds;
//                one RMAX-entry register array and a radix switch per pass);
//   CtFFT<Rs...> one plan compiled in, radices Rs in pass order: register
//                arrays of the exact radix, constant strides, divisors and
//                twiddle strides, and no switch, so each pass is straight-line
//                code of its own radix.  The launchers use it when the shot's
//                plan is one of the compiled ones (the lengths the benchmark
//                workloads and the convolution-length ladder produce).
// Both compute the same Stockham passes with the same twiddles, so their
// results agree to the last bit of the arithmetic order.
template <int RMAX> struct RtFFT {
    static constexpr int kMaxRadix = RMAX;
    static constexpr bool kCompiled = false;
    static constexpr int kLen = 0;  // the length is a run-time value
    template <int S> __device__ __forceinline__ static void run(float2* buf, int ld, const FFTCtx& c, int L) {
        fft_m_impl<S, RMAX>(buf, ld, c.sp, c.nst, c.w, L);
    }
};

// Hooks of the first and last pass of a compiled transform.  run_io lets the
// first pass take its inputs from a hook instead of the line (zero padding, a
// multiplier, another buffer) and hands the outputs of the last pass to a hook
// (a multiplier, another buffer), which folds the sweep over the line that the
// same operation costs beside a plain transform -- and that sweep's barrier --
// into the pass.  The arithmetic is the same as the separate sweep's, so the
// results agree bit for bit.  kSep: the hook reads (writes) memory other than
// the line, so that pass needs no barrier between its loads and its stores
// (no thread of the pass then loads what another one stores).
struct LineIn {
    static constexpr bool kSep = false;
    __device__ __forceinline__ float2 load(const float2* line, int i) const { return line[i]; }
};
struct LineOut {
    static constexpr bool kSep = false, kEarly = false;
    __device__ __forceinline__ void store(float2* line, int i, float2 v) const { line[i] = v; }
};
// entries [n, m) of the line read as zeros (a zero-padded convolution)
struct ZeroPadIn {
    static constexpr bool kSep = false;
    int n;
    __device__ __forceinline__ float2 load(const float2* line, int i) const {
        return (i < n) ? line[i] : make_float2(0.f, 0.f);
    }
};
// kEarly: a pure function of (i, v), applied to the outputs in registers before
// the pass's barrier (its table loads then overlap the barrier wait); the
// store after the barrier is plain.
// inputs times a complex multiplier H[i]
struct MulIn {
    static constexpr bool kSep = false;
    const float2* __restrict__ H;
    __device__ __forceinline__ float2 load(const float2* line, int i) const { return cmul(line[i], __ldg(&H[i])); }
};
// outputs times a complex multiplier H[i] (the spectrum of a convolution kernel)
struct MulOut {
    static constexpr bool kSep = false, kEarly = true;
    const float2* __restrict__ H;
    __device__ __forceinline__ float2 apply(int i, float2 v) const { return cmul(v, __ldg(&H[i])); }
    __device__ __forceinline__ void store(float2* line, int i, float2 v) const { line[i] = v; }
};
// outputs times an even real multiplier stored for 0..m/2 (tk[min(i, m - i)])
struct EvenScaleOut {
    static constexpr bool kSep = false, kEarly = true;
    const float* __restrict__ tk;
    int m;
    __device__ __forceinline__ float2 apply(int i, float2 v) const { return cscale(v, __ldg(&tk[min(i, m - i)])); }
    __device__ __forceinline__ void store(float2* line, int i, float2 v) const { line[i] = v; }
};
// outputs to another buffer (dst: this thread's line there)
struct CopyOut {
    static constexpr bool kSep = true, kEarly = false;
    float2* dst;
    __device__ __forceinline__ void store(float2*, int i, float2 v) const { dst[i] = v; }
};
// inputs from another buffer times an even real multiplier
struct EvenScaleIn {
    static constexpr bool kSep = true;
    const float2* src;
    const float* __restrict__ tk;
    int m;
    __device__ __forceinline__ float2 load(const float2*, int i) const {
        return cscale(src[i], __ldg(&tk[min(i, m - i)]));
    }
};

// Compile-time Stockham passes (NS = product of the earlier radices).  TX = 0:
// one butterfly per thread (the CTA has at least m / R threads per line for
// every pass); TX > 0: the line has TX threads and a pass of B = m / R
// butterflies gives thread j the butterflies j, j + TX, ... (NB = ceil(B / TX)
// of them), all loaded before the pass's barrier, so NB * R <= 16 keeps them
// in registers.  That is how lines longer than 768 butterflies of the smallest
// radix (m above about 5000) stay in one CTA.  The first pass loads through
// `in`, the last one stores through `out`.
template <int R, int... Rest> constexpr int first_radix() { return R; }

template <int S, int M, int NS, int TX, class In, class Out, int R, int... Rest>
__device__ __forceinline__ void ct_passes(float2* line, const float2* __restrict__ tw, bool lact, const In& in,
                                          const Out& out, float2 wpre) {
    constexpr bool kFirst = NS == 1, kLast = sizeof...(Rest) == 0;
    static_assert(!(kFirst && kLast && In::kSep && Out::kSep), "a one-pass transform between two other buffers");
    constexpr bool kSep = (kFirst && In::kSep) || (kLast && Out::kSep);
    constexpr int B = M / R;
    constexpr int NB = (TX == 0) ? 1 : (B + TX - 1) / TX;
    static_assert(NB * R <= 16, "butterflies of one thread must fit its registers");
    // One butterfly per thread (TX = 0): the next pass's twiddle is loaded at
    // the start of this pass, so its latency overlaps this pass's work and
    // barriers (the pass receives its own as wpre).
    float2 wnext = make_float2(1.f, 0.f);
    if constexpr (TX == 0 && !kLast) {
        constexpr int NS2 = NS * R, R2 = first_radix<Rest...>(), B2 = M / R2;
        const int j = threadIdx.x;
        if (lact && j < B2) wnext = __ldg(&tw[(j % NS2) * (M / (NS2 * R2))]);
    }
    float2 v[NB][R];
    int k[NB];
#pragma unroll
    for (int q = 0; q < NB; q++) {
        const int j = threadIdx.x + q * TX;
        k[q] = 0;
        if (lact && j < B) {
            if constexpr (NS > 1) k[q] = j % NS;
#pragma unroll
            for (int r = 0; r < R; r++) {
                if constexpr (kFirst) v[q][r] = in.load(line, j + r * B);
                else v[q][r] = line[j + r * B];
            }
            if constexpr (NS > 1) {
                float2 w1 = (TX == 0) ? wpre : __ldg(&tw[k[q] * (M / (NS * R))]);
                if (S > 0) w1.y = -w1.y;
                float2 w = w1;
#pragma unroll
                for (int r = 1; r < R; r++) {
                    v[q][r] = cmul(v[q][r], w);
                    w = cmul(w, w1);
                }
            }
            dft<R, S>(v[q]);
            if constexpr (kLast && Out::kEarly) {
                const int base = (j - k[q]) * R + k[q];
#pragma unroll
                for (int r = 0; r < R; r++) v[q][r] = out.apply(base + r * NS, v[q][r]);
            }
        }
    }
    if constexpr (!kSep) __syncthreads();
#pragma unroll
    for (int q = 0; q < NB; q++) {
        const int j = threadIdx.x + q * TX;
        if (lact && j < B) {
            const int base = (j - k[q]) * R + k[q];
#pragma unroll
            for (int r = 0; r < R; r++) {
                if constexpr (kLast) out.store(line, base + r * NS, v[q][r]);
                else line[base + r * NS] = v[q][r];
            }
        }
    }
    __syncthreads();
    if constexpr (!kLast) ct_passes<S, M, NS * R, TX, In, Out, Rest...>(line, tw, lact, in, out, wnext);
}

template <int TX, int... Rs> struct CtFFTX {
    static constexpr int kTX = TX;  // threads per line (0: one butterfly each)
    static constexpr int kNst = sizeof...(Rs);
    static constexpr int kRad[kNst] = {Rs...};
    static constexpr int M = (Rs * ...);
    static constexpr int kMaxRadix = [] {
        int r = 0;
        for (int x : {Rs...}) r = x > r ? x : r;
        return r;
    }();
    static constexpr bool kCompiled = true;
    static constexpr int kLen = M;
    template <int S> __device__ __forceinline__ static void run(float2* buf, int ld, const FFTCtx& c, int L) {
        ct_passes<S, M, 1, TX, LineIn, LineOut, Rs...>(buf + threadIdx.y * ld, c.w, threadIdx.y < L, LineIn{},
                                                       LineOut{}, make_float2(1.f, 0.f));
    }
    // The same transform with first- and last-pass hooks (LineIn .. EvenScaleIn
    // above).  Caller has synchronised after filling what `in` reads; ends with
    // a barrier, the result where `out` put it.
    template <int S, class In, class Out>
    __device__ __forceinline__ static void run_io(float2* buf, int ld, const FFTCtx& c, int L, const In& in,
                                                  const Out& out) {
        ct_passes<S, M, 1, TX, In, Out, Rs...>(buf + threadIdx.y * ld, c.w, threadIdx.y < L, in, out,
                                               make_float2(1.f, 0.f));
    }
    // host: is p exactly this plan (radices and, for TX > 0, threads per line)?
    static bool matches(const FFTPlanDev& p) {
        if (p.m != M || p.nst != kNst || (TX > 0 && p.tx != TX)) return false;
        for (int i = 0; i < kNst; i++)
            if (p.pass[i].R != kRad[i]) return false;
        return true;
    }
};
template <int... Rs> using CtFFT = CtFFTX<0, Rs...>;

// A list of compiled plans and its dispatch: first_match calls fn(Policy{})
// with the first listed plan that p equals and returns true, else false.
template <class... Ps> struct PlanList {};
template <class Fn> bool first_match(PlanList<>, const FFTPlanDev&, Fn&&) { return false; }
template <class P0, class... Ps, class Fn> bool first_match(PlanList<P0, Ps...>, const FFTPlanDev& p, Fn&& fn) {
    if (P0::matches(p)) {
        fn(P0{});
        return true;
    }
    return first_match(PlanList<Ps...>{}, p, fn);
}
// fn(Policy{}) for every plan of the list (e.g. to set kernel attributes)
template <class Fn> void for_each_plan(PlanList<>, Fn&&) {}
template <class P0, class... Ps, class Fn> void for_each_plan(PlanList<P0, Ps...>, Fn&& fn) {
    fn(P0{});
    for_each_plan(PlanList<Ps...>{}, fn);
}

// Launches kernel template K for plan p: a compiled plan when p is one (and
// every extra plan of the kernel equals it), else the run-time plan.
#define QP_DISPATCH(LIST, p, same_extra, r12, LAUNCH)                                  \
    do {                                                                              \
        const bool ct_ = first_match(LIST{}, p, [&](auto fp_) {                        \
            using FPc = decltype(fp_);                                                \
            if (same_extra(FPc{})) {                                                  \
                LAUNCH(FPc);                                                          \
            } else if (r12) {                                                         \
                LAUNCH(RtFFT<12>);                                                    \
            } else {                                                                  \
                LAUNCH(RtFFT<16>);                                                    \
            }                                                                         \
        });                                                                           \
        if (!ct_) {                                                                   \
            if (r12) {                                                                \
                LAUNCH(RtFFT<12>);                                                    \
            } else {                                                                  \
                LAUNCH(RtFFT<16>);                                                    \
            }                                                                         \
        }                                                                             \
    } while (0)

// QP_DISPATCH's same_extra for kernels with one plan
struct NoExtraPlan {
    template <class F> bool operator()(F) const { return true; }
};

// FP: the transform policy (RtFFT / CtFFT above)
template <int S, class FP = RtFFT<16>>
__device__ __forceinline__ void fft_m(float2* buf, int ld, const FFTCtx& pl, int L) {
    FP::template run<S>(buf, ld, pl, L);
}

// Exact length-n DFT of entries [0,n) of each line, in place.  Caller has
// synchronised after filling buf; ends with a barrier.
template <int S, class FP = RtFFT<16>>
__device__ __forceinline__ void dft_n(float2* buf, int ld, const FFTCtx& pl, int L) {
    if (!pl.blue) {
        fft_m<S, FP>(buf, ld, pl, L);
        return;
    }
    const int n = pl.n, m = pl.m;
    const int l = threadIdx.y;
    float2* line = buf + l * ld;
    const bool act = l < L;
    // inverse = conj(DFT(conj(x)))
    if (act)
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            float2 v = make_float2(0.f, 0.f);
            if (k < n) {
                float2 x = line[k];
                if (S > 0) x.y = -x.y;
                v = cmul(x, __ldg(&pl.chirp[k]));
            }
            line[k] = v;
        }
    __syncthreads();
    fft_m<-1, FP>(buf, ld, pl, L);
    if (act)
        for (int k = threadIdx.x; k < m; k += blockDim.x) line[k] = cmul(line[k], __ldg(&pl.bhat[k]));
    __syncthreads();
    fft_m<+1, FP>(buf, ld, pl, L);
    if (act)
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            float2 y = cmul(line[k], __ldg(&pl.chirp[k]));
            if (S > 0) y.y = -y.y;
            line[k] = y;
        }
    __syncthreads();
}

// Separable operator as a zero-padded circular convolution on a length-m
// plan: y[0,n) = IFFT_m(Hm .* FFT_m(x zero-padded to m)), Hm from conv_table
// (m = n when n itself is smooth).  Caller has synchronised after filling
// entries [0,n); ends with a barrier.
template <class FP = RtFFT<16>>
__device__ __forceinline__ void roundtrip_conv(float2* buf, int ld, const FFTCtx& pl, int L,
                                               const float2* __restrict__ Hm) {
    if constexpr (FP::kCompiled) {
        // zero padding folded into the first forward pass, Hm into the last
        FP::template run_io<-1>(buf, ld, pl, L, ZeroPadIn{pl.n}, MulOut{Hm});
        FP::template run<+1>(buf, ld, pl, L);
        return;
    }
    const int l = threadIdx.y;
    float2* line = buf + l * ld;
    const bool act = l < L;
    if (pl.m > pl.n) {
        if (act)
            for (int k = pl.n + threadIdx.x; k < pl.m; k += blockDim.x) line[k] = make_float2(0.f, 0.f);
        __syncthreads();
    }
    fft_m<-1, FP>(buf, ld, pl, L);
    if (act)
        for (int k = threadIdx.x; k < pl.m; k += blockDim.x) line[k] = cmul(line[k], __ldg(&Hm[k]));
    __syncthreads();
    fft_m<+1, FP>(buf, ld, pl, L);
}

// y = IDFT(H .* DFT(x)) with a complex symbol (length n, 1/n folded in).
__device__ __forceinline__ void roundtrip_c(float2* buf, int ld, const FFTCtx& pl, int L,
                                            const float2* __restrict__ H) {
    dft_n<-1>(buf, ld, pl, L);
    if (threadIdx.y < L) {
        float2* line = buf + threadIdx.y * ld;
        for (int k = threadIdx.x; k < pl.n; k += blockDim.x) line[k] = cmul(line[k], __ldg(&H[k]));
    }
    __syncthreads();
    dft_n<+1>(buf, ld, pl, L);
}

// Same with a real symbol.
__device__ __forceinline__ void roundtrip_r(float2* buf, int ld, const FFTCtx& pl, int L,
                                            const float* __restrict__ H) {
    dft_n<-1>(buf, ld, pl, L);
    if (threadIdx.y < L) {
        float2* line = buf + threadIdx.y * ld;
        for (int k = threadIdx.x; k < pl.n; k += blockDim.x) line[k] = cscale(line[k], __ldg(&H[k]));
    }
    __syncthreads();
    dft_n<+1>(buf, ld, pl, L);
}

}  // namespace qp
