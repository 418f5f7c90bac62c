// pass_common.cuh -- global<->shared movement shared by the pass kernels.
#pragma once
#include <cuda_runtime.h>

#include "qpstd_internal.h"

namespace qp {

// Asynchronous 4-byte global->shared copies (cp.async, completion per thread).
// A pass stages the inputs of its epilogues at kernel start so their loads
// overlap the FFT work; every thread later reads back only the elements it
// staged itself, so a per-thread wait (no barrier) suffices.
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// Waits for every committed group but the most recent one.
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Epilogue loops over k = k0, k0 + step, ... < n that read fields in global
// memory and write fields in global memory.  The compiler may not move a later
// iteration's loads above an earlier iteration's stores (the fields could
// alias), so each iteration would wait out the latency of its own loads.  Here
// the loads of U iterations (load(k) returns them) all issue before the first
// of their bodies (use(k, loaded)) runs; the arithmetic is unchanged.
template <int U, class LoadF, class UseF>
__device__ __forceinline__ void batched_for(int k0, int n, int step, LoadF&& load, UseF&& use) {
    using In = decltype(load(k0));
    for (int kb = k0; kb < n; kb += U * step) {
        In v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = kb + u * step;
            if (k < n) v[u] = load(k);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = kb + u * step;
            if (k < n) use(k, v[u]);
        }
    }
}
// U of the pass kernels' epilogues: x passes (one field value per point of a
// row) and z passes (two rows per point, under tighter register caps).  x
// lines of a compiled length of 2048 or more leave each thread 10 or more
// points of its tile and take 8 at a time (6 in the radix-12 instances, whose
// 48-register cap spills at 8); measured on the 5040-point lines of the large
// RTM grid: 8.8 -> 9.2 Gpts/s, the Q-RTM batch 8.37 -> 8.44.
constexpr int kEpiBatchX = 4, kEpiBatchZ = 2;
template <class FP> constexpr int x_epi_batch() { return FP::kLen < 2048 ? kEpiBatchX : FP::kMaxRadix <= 12 ? 6 : 8; }

// Compensated accumulation s += v (Kahan), used for the image and the
// illumination sums over thousands of steps.
__device__ __forceinline__ void kahan_add(float* s, float* c, size_t i, float v) {
    const float y = v - c[i];
    const float t = s[i] + y;
    c[i] = (t - s[i]) - y;
    s[i] = t;
}
// The same with s[i], c[i] already loaded (s0, c0).
__device__ __forceinline__ void kahan_add_v(float* s, float* c, size_t i, float s0, float c0, float v) {
    const float y = v - c0;
    const float t = s0 + y;
    c[i] = (t - s0) - y;
    s[i] = t;
}

// z passes: this thread's line packs x rows r0 (re) and r1 (im); 4 points'
// loads at a time (only registers for the loaded pair are held, so the z
// passes' cap allows it: measured ahead of 2, 8.39 against 8.33 Gpts/s).
__device__ __forceinline__ void zload_pair(const float* __restrict__ f, float2* line, int nzz, bool has0, bool has1,
                                           size_t r0, size_t r1) {
    batched_for<kEpiBatchX>(
        threadIdx.x, nzz, blockDim.x,
        [&](int k) { return make_float2(has0 ? f[r0 + k] : 0.f, has1 ? f[r1 + k] : 0.f); },
        [&](int k, float2 v) { line[k] = v; });
}

// Half spectra in kz: S[ix*nzh + kz], kz in [0, nzz/2].  Two real z-lines a, b
// share one complex line z = a + ib: A(k) = (Z(k) + conj Z(n-k))/2,
// B(k) = (Z(k) - conj Z(n-k))/(2i), and back Z(k) = A(k) + iB(k).
// this thread's packed line <- half spectra of rows (xa, xa+1)
__device__ __forceinline__ void zrepack(const float2* __restrict__ S, float2* line, int nzz, int nzh, bool has0,
                                        bool has1, int xa) {
    for (int k = threadIdx.x; k < nzz; k += blockDim.x) {
        const int kk = (k < nzh) ? k : nzz - k;
        const float2 A = has0 ? S[(size_t)xa * nzh + kk] : make_float2(0.f, 0.f);
        const float2 B = has1 ? S[(size_t)(xa + 1) * nzh + kk] : make_float2(0.f, 0.f);
        line[k] = (k < nzh) ? make_float2(A.x - B.y, A.y + B.x) : make_float2(A.x + B.y, -A.y + B.x);
    }
}

// zrepack as the load hook of a compiled transform's first pass (fft_reg.cuh,
// run_io): entry k of the packed line, read straight from the half spectra.
struct ZRepackIn {
    static constexpr bool kSep = true;
    const float2* __restrict__ S;
    int nzz, nzh, xa;
    bool has0, has1;
    __device__ __forceinline__ float2 load(const float2*, int k) const {
        const int kk = (k < nzh) ? k : nzz - k;
        const float2 A = has0 ? S[(size_t)xa * nzh + kk] : make_float2(0.f, 0.f);
        const float2 B = has1 ? S[(size_t)(xa + 1) * nzh + kk] : make_float2(0.f, 0.f);
        return (k < nzh) ? make_float2(A.x - B.y, A.y + B.x) : make_float2(A.x + B.y, -A.y + B.x);
    }
};

// half spectra of rows (xa, xa+1) <- this thread's transformed packed line
__device__ __forceinline__ void zunpack(const float2* line, float2* __restrict__ S, int nzz, int nzh, bool has0,
                                        bool has1, int xa) {
    for (int k = threadIdx.x; k < nzh; k += blockDim.x) {
        const float2 z = line[k];
        const float2 w = line[(k == 0) ? 0 : nzz - k];
        if (has0) S[(size_t)xa * nzh + k] = make_float2(0.5f * (z.x + w.x), 0.5f * (z.y - w.y));
        if (has1) S[(size_t)(xa + 1) * nzh + k] = make_float2(0.5f * (z.y + w.y), -0.5f * (z.x - w.x));
    }
}

// x passes: a CTA owns TZ = 2L consecutive z columns (TZ a power of two); line
// l holds columns (iz0+2l, iz0+2l+1) in re/im, indexed by x.  Global accesses
// walk (ix, c) with c fastest so each x row is read as one TZ-float segment.
struct XTile {
    int iz0, tzlog, tot, t0, nthr, nzz;
    __device__ __forceinline__ XTile(int L, int bx, int nzz_, int nxx) {
        const int TZ = 2 * L;
        tzlog = 31 - __clz(TZ);
        iz0 = bx * TZ;
        tot = nxx * TZ;
        t0 = threadIdx.y * blockDim.x + threadIdx.x;
        nthr = blockDim.x * blockDim.y;
        nzz = nzz_;
    }
    __device__ __forceinline__ void split(int g, int& c, int& ix) const {
        c = g & ((1 << tzlog) - 1);
        ix = g >> tzlog;
    }
    // float index of (column c, position ix) in the packed shared lines
    __device__ __forceinline__ int sidx(int c, int ix, int ld) const { return 2 * ((c >> 1) * ld + ix) + (c & 1); }
};

// the packed shared lines <- get(g, ix, iz) for the tile's columns (0 past nzz),
// a group of points' loads in flight at a time
template <int U, class Get>
__device__ __forceinline__ void xfill(float* sf, const XTile& T, int ld, Get&& get) {
    batched_for<U>(
        T.t0, T.tot, T.nthr,
        [&](int g) {
            int c, ix;
            T.split(g, c, ix);
            const int iz = T.iz0 + c;
            return (iz < T.nzz) ? get(g, ix, iz) : 0.f;
        },
        [&](int g, float v) {
            int c, ix;
            T.split(g, c, ix);
            sf[T.sidx(c, ix, ld)] = v;
        });
}

}  // namespace qp
