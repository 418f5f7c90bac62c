// host_setup.cpp -- one-time FP64 coefficient setup and line-FFT plans.
//
// The reference computes its coefficient tables on the host in float
// (sgpstd-qmodeling/funca.c, func.c); here every table is evaluated in double
// and rounded once to float.  The formulas are the reference's:
//   CPML profiles            funca.c:223-340  (get_pml_parameters)
//   half-cell shift symbols  funca.c:342-432  (cal_shift_parameters)
//   wavenumbers              funca.c:366-381 / func.c:550-585 (cal_k2d)
// including the reference's pi = 3.1415926 and its mirror index n/2*2-i for the
// negative-frequency shift phases.
#include "host_setup.h"

#include <initializer_list>

#include "xplans_list.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

namespace qp {

static const double REF_PI = 3.1415926;  // funca.c:6

void pml_coeffs(int pml, double fm, int nxx, int nzz, double dx, double dz, double dt, std::vector<double>* out8) {
    const double alpha_max = REF_PI * fm, R = 1e-5, vmax = 5000.0;
    const int n1 = 2, n2 = 1, n3 = 1;
    std::vector<double> idx(nxx), idz(nzz), iax(nxx), iaz(nzz), hdx(nxx), hdz(nzz), hax(nxx), haz(nzz);
    const double dmaxx = (1 + n1 + n2) * vmax * std::log(1.0 / R) / (2.0 * pml * dx);
    const double dmaxz = (1 + n1 + n2) * vmax * std::log(1.0 / R) / (2.0 * pml * dz);
    for (int i = 0; i < pml; i++) {
        const double t1 = std::pow((double)(pml - 1 - i) / pml, n1 + n2);
        const double t3 = std::pow((double)i / (pml - 1), n3);
        idx[i] = dmaxx * t1;
        idz[i] = dmaxz * t1;
        iax[i] = alpha_max * t3;
        iaz[i] = iax[i];
        idx[nxx - 1 - i] = idx[i];
        idz[nzz - 1 - i] = idz[i];
        iax[nxx - 1 - i] = iax[i];
        iaz[nzz - 1 - i] = iaz[i];
    }
    for (int i = pml; i < nxx - pml; i++) { idx[i] = 0; iax[i] = iax[pml - 1]; }
    for (int j = pml; j < nzz - pml; j++) { idz[j] = 0; iaz[j] = iaz[pml - 1]; }
    for (int i = 0; i < pml - 1; i++) {
        const double t2 = std::pow((pml - 1.5 - i) / pml, n1 + n2);
        const double t4 = std::pow((i + 0.5) / (pml - 1), n3);
        hdx[i] = dmaxx * t2;
        hdz[i] = dmaxz * t2;
        hdx[nxx - 2 - i] = hdx[i];
        hdz[nzz - 2 - i] = hdz[i];
        hax[i] = alpha_max * t4;
        haz[i] = hax[i];
        hax[nxx - 2 - i] = hax[i];
        haz[nzz - 2 - i] = haz[i];
    }
    for (int i = pml - 1; i < nxx - pml; i++) { hdx[i] = 0; hax[i] = hax[pml - 2]; }
    hdx[nxx - 1] = 0;
    hax[nxx - 1] = hax[nxx - 2];
    for (int j = pml - 1; j < nzz - pml; j++) { hdz[j] = 0; haz[j] = haz[pml - 2]; }
    hdz[nzz - 1] = 0;
    haz[nzz - 1] = haz[nzz - 2];
    // order: i_ax, i_bx, i_az, i_bz, h_ax, h_bx, h_az, h_bz
    for (int k = 0; k < 8; k++) out8[k].assign((k % 4 < 2) ? nxx : nzz, 0.0);
    for (int i = 0; i < nxx; i++) {
        double t = idx[i] + iax[i];
        out8[1][i] = std::exp(-dt * t);
        out8[0][i] = idx[i] / t * (out8[1][i] - 1.0);
        t = hdx[i] + hax[i];
        out8[5][i] = std::exp(-dt * t);
        out8[4][i] = hdx[i] / t * (out8[5][i] - 1.0);
    }
    for (int j = 0; j < nzz; j++) {
        double t = idz[j] + iaz[j];
        out8[3][j] = std::exp(-dt * t);
        out8[2][j] = idz[j] / t * (out8[3][j] - 1.0);
        t = hdz[j] + haz[j];
        out8[7][j] = std::exp(-dt * t);
        out8[6][j] = hdz[j] / t * (out8[7][j] - 1.0);
    }
}

double wavenumber(int i, int n, double d) {
    const double dk = 2.0 * REF_PI / (n * d);
    return (i < n / 2 + 1) ? i * dk : (n - i) * dk;
}

// Reference symbol of shift_vxz_kernel / shift_pxz_kernel at index i
// (acps4.cu:1047-1108): the kernels form H = -b + i a for i < n/2+1 and
// H = b - i a above, from the table pair (a, b).
static std::complex<double> ref_symbol(double a, double b, int i, int n) {
    return (i < n / 2 + 1) ? std::complex<double>(-b, a) : std::complex<double>(b, -a);
}

void shift_symbols(int n, double d, int which, std::vector<std::complex<double>>& H, bool raw) {
    // which: 0 = "m" tables used for the velocity derivative along x
    //            (kxsmr, kxsmi) ; 1 = "c" tables used for the pressure
    //            derivative along x (kxscr, kxsci) ; 2 = z velocity derivative
    //            (kzscr, kzsci) ; 3 = z pressure derivative (kzsmr, kzsmi)
    std::vector<double> sr(n), si(n), a(n), b(n);
    const int nh = n / 2 + 1;
    for (int i = 0; i < n; i++) {
        if (i < nh) {
            const double t = i * REF_PI / n;
            sr[i] = std::cos(t);
            si[i] = std::sin(t);
        } else {
            sr[i] = sr[n / 2 * 2 - i];
            si[i] = -si[n / 2 * 2 - i];
        }
        const double k = wavenumber(i, n, d);
        switch (which) {
            case 0: a[i] = k * sr[i]; b[i] = -k * si[i]; break;  // kxsmr, kxsmi
            case 1: a[i] = k * sr[i]; b[i] = k * si[i]; break;   // kxscr, kxsci
            case 2: a[i] = k * sr[i]; b[i] = -k * si[i]; break;  // kzscr, kzsci
            default: a[i] = k * sr[i]; b[i] = k * si[i]; break;  // kzsmr, kzsmi
        }
    }
    if (raw) {
        // the reference's own symbol, as multiplied inside its 2-D C2C path
        H.assign(n, 0.0);
        for (int i = 0; i < n; i++) H[i] = ref_symbol(a[i], b[i], i, n);
        return;
    }
    // The reference keeps Re of a C2C inverse of real data, i.e. it applies the
    // Hermitian part (H(k) + conj(H(-k)))/2 of its symbol.  For odd n the
    // mirrored phases make H itself non-Hermitian, so the effective symbol is
    // formed explicitly; the 1/n of the line transform is folded in.
    H.assign(n, 0.0);
    for (int i = 0; i < n; i++) {
        const std::complex<double> h = ref_symbol(a[i], b[i], i, n);
        const int j = (n - i) % n;
        const std::complex<double> hm = ref_symbol(a[j], b[j], j, n);
        H[i] = 0.5 * (h + std::conj(hm)) / (double)n;
    }
}

// ---- FFT plans --------------------------------------------------------------
static bool smooth7(int v) {
    for (int f : {2, 3, 5, 7})
        while (v % f == 0) v /= f;
    return v == 1;
}

// Radices of the register passes (each 2..16): fewest passes first, then the
// largest smallest radix, since a pass of radix R keeps m/R threads per line
// busy (5184 -> 9,9,8,8 runs on 648 threads; 1728 -> 12,12,12 on 144), then
// the smaller largest radix (a plan with radices up to 12 runs the kernels'
// 12-entry register array, in fewer registers).
static void factor_search(int v, int maxr, std::vector<int>& cur, std::vector<int>& best) {
    if (v == 1) {
        if (best.empty() || cur.size() < best.size()) {
            best = cur;
        } else if (cur.size() == best.size()) {
            const int cmin = *std::min_element(cur.begin(), cur.end());
            const int bmin = *std::min_element(best.begin(), best.end());
            const int cmax = *std::max_element(cur.begin(), cur.end());
            const int bmax = *std::max_element(best.begin(), best.end());
            if (cmin > bmin || (cmin == bmin && cmax < bmax)) best = cur;
        }
        return;
    }
    if (!best.empty() && cur.size() + 1 > best.size()) return;
    for (int r = std::min(maxr, 16); r >= 2; r--) {
        if (v % r) continue;
        cur.push_back(r);
        factor_search(v / r, r, cur, best);  // non-increasing radices: each multiset once
        cur.pop_back();
    }
}

// Relative cost of a length whose plan has radices up to 12: the pass kernels
// then run at 48 instead of 56 registers per thread (qpstd_internal.h), which
// is worth a slightly longer transform when several lengths are admissible.
static double radix_weight(const std::vector<int>& rad) {
    return (*std::max_element(rad.begin(), rad.end()) <= 12) ? 0.85 : 1.0;
}

static bool factor_direct(int n, std::vector<int>& rad) {
    rad.clear();
    if (n > 65535) return false;
    std::vector<int> cur;
    factor_search(n, 16, cur, rad);
    if (rad.empty() || (int)rad.size() > QP_MAXST) return false;
    // odd radices first: the first pass writes at stride R, which is free of
    // shared-memory bank conflicts only for odd R (measured: -12 % step time on a
    // 1678-wide Q-RTM shot, whose 3360 = 16*15*14 convolution length runs 15,16,14)
    std::stable_partition(rad.begin(), rad.end(), [](int r) { return r % 2 == 1; });
    const int rmin = *std::min_element(rad.begin(), rad.end());
    return n / rmin <= QP_MAXTHREADS;
}

// Host Stockham in double (same recurrence as the device engine).
static void host_fft(std::vector<std::complex<double>>& x, const std::vector<int>& rad, int sgn) {
    const int n = (int)x.size();
    std::vector<std::complex<double>> y(n);
    std::vector<std::complex<double>>*src = &x, *dst = &y;
    int ns = 1;
    for (int r : rad) {
        const int nb = n / r;
        for (int j = 0; j < nb; j++) {
            const int k = j % ns;
            std::complex<double> v[16], o[16];
            for (int q = 0; q < r; q++) {
                const double ang = sgn * 2.0 * M_PI * (double)(q * k) / (double)(ns * r);
                v[q] = (*src)[j + q * nb] * std::complex<double>(std::cos(ang), std::sin(ang));
            }
            for (int q = 0; q < r; q++) {
                std::complex<double> acc = 0;
                for (int u = 0; u < r; u++) {
                    const double ang = sgn * 2.0 * M_PI * (double)((u * q) % r) / (double)r;
                    acc += v[u] * std::complex<double>(std::cos(ang), std::sin(ang));
                }
                o[q] = acc;
            }
            const int base = (j - k) * r + k;
            for (int q = 0; q < r; q++) (*dst)[base + q * ns] = o[q];
        }
        std::swap(src, dst);
        ns *= r;
    }
    if (src != &x) x = *src;
}

// Lengths whose x passes are compiled with the plan built in (xplans_list.h):
// their passes run about a fifth faster than the run-time plan (measured on
// the z passes), which the planner counts as a lower cost.  Long entries
// (TX > 0) are the only plans for lines beyond the one-butterfly-per-thread
// limit.
struct CompiledPlan {
    int tx;
    std::vector<int> rad;
    int m() const {
        int v = 1;
        for (int r : rad) v *= r;
        return v;
    }
};
#define QP_XPLAN_ENTRY(TX, ...) CompiledPlan{TX, {__VA_ARGS__}},
static const std::vector<CompiledPlan>& compiled_plans() {
    static const std::vector<CompiledPlan> v = {QP_XPLANS_ALL(QP_XPLAN_ENTRY)};
    return v;
}
static const CompiledPlan* compiled_length(int m) {
    for (const CompiledPlan& c : compiled_plans())
        if (c.m() == m) return &c;
    return nullptr;
}
static bool compiled_conv_length(int m) {
    const CompiledPlan* c = compiled_length(m);
    return c && c->tx == 0;
}

// The smooth lengths m in [2n-1, 2.3n+8] a zero-padded convolution or a
// Bluestein transform of an n-point line can use, with their radices: the
// cheapest by pass work (extra_pass: 1 for Bluestein's two transforms per
// DFT), compiled plans counted at 0.8; with allow_long, a compiled long plan
// when no length has a one-butterfly-per-thread plan.
static bool choose_inner_length(int n, bool allow_long, int extra_pass, HostPlan& hp) {
    double best = 1e300;
    for (int m = 2 * n - 1; m <= (int)(2.3 * n) + 8; m++) {
        if (!smooth7(m)) continue;
        std::vector<int> r;
        if (!factor_direct(m, r)) continue;
        double cost = (double)m * (r.size() + extra_pass) * radix_weight(r);
        if (compiled_conv_length(m)) cost *= 0.8;
        if (cost < best) {
            best = cost;
            hp.m = m;
            hp.rad = r;
            hp.tx = 0;
        }
    }
    if (best < 1e300 || !allow_long) return best < 1e300;
    for (int m = 2 * n - 1; m <= (int)(2.3 * n) + 8; m++) {
        const CompiledPlan* c = compiled_length(m);
        if (!c || c->tx == 0) continue;
        hp.m = m;
        hp.rad = c->rad;
        hp.tx = c->tx;
        return true;
    }
    return false;
}

int build_plan_host(int n, HostPlan& hp, bool allow_long) {
    hp.n = n;
    hp.blue = 0;
    hp.tx = 0;
    if (n == 1) {
        hp.m = 1;
        hp.rad.clear();
    } else if (factor_direct(n, hp.rad)) {
        hp.m = n;
    } else {
        // Bluestein: the {2,3,5,7}-smooth inner length in [2n-1, 2.3n] with the
        // lowest pass work, m * (passes + 1), weighted by radix_weight; for long
        // lines the compiled long plan the convolution plan of n takes too
        hp.blue = 1;
        if (!choose_inner_length(n, allow_long, 1, hp)) return -1;
        if (hp.tx > 0) {
            HostPlan c;
            if (build_conv_plan_host(n, c, true) || c.tx == 0) return -1;
            hp.m = c.m;
            hp.rad = c.rad;
            hp.tx = c.tx;
        }
    }
    const int m = hp.m;
    hp.w.resize(m);
    for (int k = 0; k < m; k++) {
        const double a = -2.0 * M_PI * (double)k / (double)m;
        hp.w[k] = std::complex<double>(std::cos(a), std::sin(a));
    }
    hp.chirp.clear();
    hp.bhat.clear();
    if (hp.blue) {
        hp.chirp.resize(n);
        for (long long k = 0; k < n; k++) {
            const long long q = (k * k) % (2LL * n);
            const double a = -M_PI * (double)q / (double)n;
            hp.chirp[k] = std::complex<double>(std::cos(a), std::sin(a));
        }
        std::vector<std::complex<double>> b(m, 0.0);
        for (int k = 0; k < n; k++) b[k] = std::conj(hp.chirp[k]);
        for (int k = 1; k < n; k++) b[m - k] = std::conj(hp.chirp[k]);
        host_fft(b, hp.rad, -1);
        hp.bhat.resize(m);
        for (int k = 0; k < m; k++) hp.bhat[k] = b[k] / (double)m;
    }
    return 0;
}

// A separable spectral operator y = IDFT_n(H . DFT_n(x)) is the circular
// convolution of x with h = IDFT_n(H).  Any length m >= 2n-1 computes it with
// one zero-padded forward and one inverse length-m FFT (every lag i-j in
// (-n, n) lands on a distinct slot of the length-m wrap), so a window length
// with a large prime factor costs two smooth FFTs instead of Bluestein's four.
int build_conv_plan_host(int n, HostPlan& hp, bool allow_long) {
    hp = HostPlan();
    hp.n = n;
    if (n == 1 || factor_direct(n, hp.rad)) {
        hp.m = (n == 1) ? 1 : n;
        if (n == 1) hp.rad.clear();
    } else if (!choose_inner_length(n, allow_long, 0, hp)) {
        return -1;
    }
    hp.w.resize(hp.m);
    for (int k = 0; k < hp.m; k++) {
        const double a = -2.0 * M_PI * (double)k / (double)hp.m;
        hp.w[k] = std::complex<double>(std::cos(a), std::sin(a));
    }
    return 0;
}

// Spectrum (length m, 1/m folded in) of the zero-padded, wrapped kernel of the
// operator whose length-n symbol is Hn (1/n already folded in).
void conv_table(const HostPlan& hp, const std::vector<std::complex<double>>& Hn,
                std::vector<std::complex<double>>& out) {
    const int n = hp.n, m = hp.m;
    if (m == n) {
        out = Hn;
        return;
    }
    // h[d] = sum_k Hn[k] e^{+2 pi i k d / n}, exact phases from (k d) mod n
    std::vector<std::complex<double>> h(n), e(n);
    for (int q = 0; q < n; q++) e[q] = std::complex<double>(std::cos(2.0 * M_PI * q / n), std::sin(2.0 * M_PI * q / n));
    for (int d = 0; d < n; d++) {
        std::complex<double> acc = 0.0;
        for (int k = 0; k < n; k++) acc += Hn[k] * e[(int)(((long long)k * d) % n)];
        h[d] = acc;
    }
    std::vector<std::complex<double>> hm(m, 0.0);
    for (int d = 0; d < n; d++) hm[d] = h[d];               // lags 0 .. n-1
    for (int d = 1; d < n; d++) hm[m - d] = h[n - d];       // lags -(n-1) .. -1
    host_fft(hm, hp.rad, -1);
    out.resize(m);
    for (int k = 0; k < m; k++) out[k] = hm[k] / (double)m;
}

int fill_plan_dev(const HostPlan& hp, FFTPlanDev& d) {
    d.n = hp.n;
    d.m = hp.m;
    d.blue = hp.blue;
    d.nst = (int)hp.rad.size();
    int ns = 1, maxb = 1;
    for (int i = 0; i < d.nst; i++) {
        FFTPass& p = d.pass[i];
        p.R = hp.rad[i];
        p.ns = ns;
        p.B = hp.m / p.R;
        p.twstride = hp.m / (ns * p.R);
        p.ns_magic = (ns > 1) ? (unsigned)(((1ull << 32) + ns - 1) / ns) : 0u;
        maxb = std::max(maxb, p.B);
        ns *= p.R;
    }
    d.w = d.chirp = d.bhat = nullptr;
    if (hp.tx > 0) {  // a compiled long plan: TX threads, several butterflies each
        d.tx = hp.tx;
        return 0;
    }
    d.tx = std::min(QP_MAXTHREADS, (maxb + 31) / 32 * 32);
    return (maxb > QP_MAXTHREADS) ? -1 : 0;
}

void plan_tables(const HostPlan& hp, std::vector<float2>& out) {
    out.clear();
    out.reserve(hp.w.size() + hp.chirp.size() + hp.bhat.size());
    for (auto& c : hp.w) out.push_back(make_float2((float)c.real(), (float)c.imag()));
    for (auto& c : hp.chirp) out.push_back(make_float2((float)c.real(), (float)c.imag()));
    for (auto& c : hp.bhat) out.push_back(make_float2((float)c.real(), (float)c.imag()));
}

int choose_L(int nlines, int m, int tx, int nbuf, bool pow2, size_t extra_per_line, size_t budget) {
    const size_t per_line = (size_t)8 * m * nbuf + extra_per_line;
    const int lmax = std::max(1, std::min(QP_MAXTHREADS / tx, (int)(budget / per_line)));
    int L = (nlines + 2 * 152 - 1) / (2 * 152);
    L = std::max(1, std::min(L, lmax));
    if (pow2) {
        int p = 1;
        while (p * 2 <= L) p *= 2;
        L = p;
    }
    return L;
}

}  // namespace qp
