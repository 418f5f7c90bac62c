// host_setup.h -- FP64 coefficient setup and line-FFT plan construction.
#pragma once
#include <complex>
#include <vector>

#include "qpstd_internal.h"

namespace qp {

// CPML coefficients; out8 = i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz.
void pml_coeffs(int pml, double fm, int nxx, int nzz, double dx, double dz, double dt, std::vector<double>* out8);

// |k| on an n-point grid as the reference builds it (kkx / kkz).
double wavenumber(int i, int n, double d);

// Effective (Hermitian) staggered-derivative symbol divided by n, or with
// raw=true the reference's own (unnormalised, possibly non-Hermitian) symbol.
// which: 0 = x velocity derivative, 1 = x pressure derivative,
//        2 = z velocity derivative, 3 = z pressure derivative.
void shift_symbols(int n, double d, int which, std::vector<std::complex<double>>& H, bool raw = false);

struct HostPlan {
    int n = 0, m = 0, blue = 0;
    int tx = 0;  // threads per line of a compiled long plan (0: one butterfly per thread)
    std::vector<int> rad;
    std::vector<std::complex<double>> w, chirp, bhat;
};
// allow_long: lines that only a compiled long plan (xplans_list.h, group 3)
// can run may use one; only the x passes have those kernels.
int build_plan_host(int n, HostPlan& hp, bool allow_long = false);
// Length-m FFT plan for separable operators applied as zero-padded circular
// convolutions (m = n when n factors into radices <= 16, else smooth m >= 2n-1).
int build_conv_plan_host(int n, HostPlan& hp, bool allow_long = false);
// Length-m multiplier of the convolution form of the symbol Hn (1/n folded in).
void conv_table(const HostPlan& hp, const std::vector<std::complex<double>>& Hn,
                std::vector<std::complex<double>>& out);

// Device view of a plan without its tables: passes, thread count per line.
// Returns -1 when a pass needs more threads per line than a CTA holds.
int fill_plan_dev(const HostPlan& hp, FFTPlanDev& d);
// The plan's tables in device order: twiddles, then (Bluestein) chirp and bhat.
void plan_tables(const HostPlan& hp, std::vector<float2>& out);

// Complex lines per CTA: bounded by the CTA's threads (tx per line), by shared
// memory (nbuf line buffers of m float2, plus extra_per_line bytes), and small
// enough that the grid covers the 152 SMs about twice.  pow2: a power of two.
int choose_L(int nlines, int m, int tx, int nbuf, bool pow2, size_t extra_per_line = 0,
             size_t budget = 160 * 1024);

}  // namespace qp
