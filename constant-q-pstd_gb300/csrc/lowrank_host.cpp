// lowrank_host.cpp -- FP64 low-rank decomposition of the mixed-domain
// constant-Q symbol (the one-time setup of the low-rank form).
//
// The steps of acsglowrank2d (sgpstd-qmodeling/sglowrank.c:148-480):
//  1. mm = (int)(col ln N1) random points; Sr = W(points, every k)   (:156-186)
//  2. col greedy steps over the wavenumbers: take the column of Sr with the
//     largest norm among those not taken yet; unless it is the last step,
//     keep it and remove from every remaining column its projections on all
//     kept columns, one after another (:188-244).  U = W(every point, the
//     chosen wavenumbers jrr)  (N1 x col, :247-258).
//  3. nn = (int)(row ln N2) random wavenumbers; the same greedy selection over
//     the points (:274-383); V = W(the chosen points irr, every k)  (:387-399).
//  4. np = min(mm, nn) random points r3 and wavenumbers r4; A = pinv(U[r3,:])
//     W(r3, r4) pinv(V[:, r4])  (col x row, :409-453).
// Where this differs from the reference: everything is FP64 (the reference
// samples W in float); one seeded splitmix64 generator replaces the four
// srand(time)/rand() draws, so a decomposition is reproducible; a greedy step
// that finds no candidate of positive norm takes the first one not taken (the
// reference keeps index 0, or indexes flag2[-1]); the pseudo-inverse is taken
// from a one-sided Jacobi SVD with singular values at or below 1e-8 sigma_max
// dropped (the reference calls ginv from 4GINV.C, which is not in its tree,
// with eps = 1e-8).
#include <algorithm>
#include <cmath>
#include <thread>

#include "host_setup.h"
#include "lowrank.h"

namespace qp {

double lowrank_symbol(double vp, double gam, double tao, double dt, double k) {
    const double u = 0.5 * vp * dt * std::pow(k, 1.0 + gam);
    const double sinc = (u == 0.0) ? 1.0 : std::sin(u) / u;
    return sinc * std::pow(k, gam) * std::sqrt(1.0 + 0.5 * dt * tao * std::pow(k, 1.01));
}

void lowrank_khalf(int nxx, int nzz, double dx, double dz, std::vector<double>& k) {
    const int nxh = nxx / 2 + 1, nzh = nzz / 2 + 1;
    k.assign((size_t)nxh * nzh, 0.0);
    for (int i = 0; i < nxh; i++) {
        const double kx = wavenumber(i, nxx, dx);
        for (int j = 0; j < nzh; j++) {
            const double kz = wavenumber(j, nzz, dz);
            k[(size_t)i * nzh + j] = std::sqrt(kx * kx + kz * kz);
        }
    }
    k[0] = 1.0e-6;
}

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
};

// count distinct values in [0, n), drawn in order (random_select, sglowrank.c:5-22)
std::vector<int> draw_distinct(SplitMix64& g, int n, int count) {
    count = std::min(count, n);
    std::vector<int> out;
    std::vector<char> seen(n, 0);
    while ((int)out.size() < count) {
        const int v = (int)(g.next() % (uint64_t)n);
        if (!seen[v]) {
            seen[v] = 1;
            out.push_back(v);
        }
    }
    return out;
}

template <class F> void parallel_for(size_t n, F f) {
    const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || hw == 1) {
        for (size_t i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> th;
    const size_t chunk = (n + hw - 1) / hw;
    for (unsigned t = 0; t < hw; t++) {
        const size_t a = t * chunk, b = std::min(n, a + chunk);
        if (a >= b) break;
        th.emplace_back([=, &f] {
            for (size_t i = a; i < b; i++) f(i);
        });
    }
    for (auto& x : th) x.join();
}

// Greedy selection over candidates stored contiguously (candidate c at
// S[c*len .. c*len+len)); S is deflated in place.
std::vector<int> greedy_select(std::vector<double>& S, int ncand, int len, int count) {
    std::vector<char> taken(ncand, 0);
    std::vector<int> chosen(count, 0);
    std::vector<std::vector<double>> kept;
    std::vector<double> nrm(ncand);
    for (int n = 0; n < count; n++) {
        parallel_for(ncand, [&](size_t c) {
            double s = 0.0;
            const double* v = &S[c * len];
            for (int i = 0; i < len; i++) s += v[i] * v[i];
            nrm[c] = s;
        });
        double mx = 0.0;
        int pick = -1;
        for (int c = 0; c < ncand; c++)
            if (!taken[c] && nrm[c] - mx > 0.0) {
                mx = nrm[c];
                pick = c;
            }
        if (pick < 0)
            for (int c = 0; c < ncand && pick < 0; c++)
                if (!taken[c]) pick = c;
        if (pick < 0) break;
        chosen[n] = pick;
        taken[pick] = 1;
        if (n == count - 1) break;
        kept.emplace_back(S.begin() + (size_t)pick * len, S.begin() + (size_t)pick * len + len);
        std::vector<double> kk(kept.size());
        for (size_t b = 0; b < kept.size(); b++) {
            double s = 0.0;
            for (int i = 0; i < len; i++) s += kept[b][i] * kept[b][i];
            kk[b] = s;
        }
        parallel_for(ncand, [&](size_t c) {
            if (taken[c]) return;
            double* v = &S[c * len];
            for (size_t b = 0; b < kept.size(); b++) {
                if (kk[b] == 0.0) continue;
                double d = 0.0;
                for (int i = 0; i < len; i++) d += kept[b][i] * v[i];
                const double t = d / kk[b];
                for (int i = 0; i < len; i++) v[i] -= t * kept[b][i];
            }
        });
    }
    return chosen;
}

// one-sided Jacobi SVD of the m x n (m >= n) row-major G: on return the
// columns of G are U_j sigma_j and Vm (n x n) holds V.
void jacobi_svd(std::vector<double>& G, int m, int n, std::vector<double>& Vm) {
    Vm.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) Vm[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 80; sweep++) {
        bool rotated = false;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int i = 0; i < m; i++) {
                    const double gp = G[(size_t)i * n + p], gq = G[(size_t)i * n + q];
                    al += gp * gp;
                    be += gq * gq;
                    ga += gp * gq;
                }
                if (ga == 0.0 || std::fabs(ga) <= 1e-15 * std::sqrt(al * be)) continue;
                rotated = true;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < m; i++) {
                    double& gp = G[(size_t)i * n + p];
                    double& gq = G[(size_t)i * n + q];
                    const double a = gp, b = gq;
                    gp = c * a - s * b;
                    gq = s * a + c * b;
                }
                for (int i = 0; i < n; i++) {
                    double& vp = Vm[(size_t)i * n + p];
                    double& vq = Vm[(size_t)i * n + q];
                    const double a = vp, b = vq;
                    vp = c * a - s * b;
                    vq = s * a + c * b;
                }
            }
        if (!rotated) break;
    }
}

}  // namespace

void pinv(const std::vector<double>& M, int m, int n, double eps, std::vector<double>& P) {
    if (m < n) {  // pinv(M) = pinv(M^T)^T
        std::vector<double> T((size_t)n * m), PT;
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) T[(size_t)j * m + i] = M[(size_t)i * n + j];
        pinv(T, n, m, eps, PT);  // m x n
        P.assign((size_t)n * m, 0.0);
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) P[(size_t)j * m + i] = PT[(size_t)i * n + j];
        return;
    }
    std::vector<double> G = M, Vm;
    jacobi_svd(G, m, n, Vm);
    std::vector<double> s2(n, 0.0);
    double smax = 0.0;
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < m; i++) s2[j] += G[(size_t)i * n + j] * G[(size_t)i * n + j];
        smax = std::max(smax, std::sqrt(s2[j]));
    }
    // P = V diag(1/sigma) U^T = sum_j V[:,j] (G[:,j] / sigma_j^2)^T
    P.assign((size_t)n * m, 0.0);
    for (int j = 0; j < n; j++) {
        if (!(std::sqrt(s2[j]) > eps * smax)) continue;
        for (int a = 0; a < n; a++) {
            const double va = Vm[(size_t)a * n + j] / s2[j];
            if (va == 0.0) continue;
            for (int i = 0; i < m; i++) P[(size_t)a * m + i] += va * G[(size_t)i * n + j];
        }
    }
}

int lowrank_decompose(int nxx, int nzz, double dx, double dz, double dt, const float* vp, const float* tao,
                      const float* gam, int row, int col, uint64_t seed, LowRankFactors& f) {
    const int N1 = nxx * nzz;
    const int nxh = nxx / 2 + 1, nzh = nzz / 2 + 1, N2 = nxh * nzh;
    std::vector<double> k;
    lowrank_khalf(nxx, nzz, dx, dz, k);
    auto W = [&](int x, int j) { return lowrank_symbol(vp[x], gam[x], tao[x], dt, k[j]); };
    SplitMix64 g{seed};

    // 1-2: wavenumber columns (Sr stored wavenumber-major: column j at j*mm)
    const int mm = std::min(N1, (int)(col * std::log((double)N1)));
    const std::vector<int> r1 = draw_distinct(g, N1, mm);
    std::vector<double> Sr((size_t)N2 * mm);
    parallel_for(N2, [&](size_t j) {
        for (int i = 0; i < mm; i++) Sr[j * mm + i] = W(r1[i], (int)j);
    });
    f.jrr = greedy_select(Sr, N2, mm, col);
    Sr.clear();
    Sr.shrink_to_fit();
    f.U.assign((size_t)N1 * col, 0.f);
    parallel_for(N1, [&](size_t x) {
        for (int a = 0; a < col; a++) f.U[x * col + a] = (float)W((int)x, f.jrr[a]);
    });

    // 3: point rows (Sc point-major: point i at i*nn)
    const int nn = std::min(N2, (int)(row * std::log((double)N2)));
    const std::vector<int> r2 = draw_distinct(g, N2, nn);
    std::vector<double> Sc((size_t)N1 * nn);
    parallel_for(N1, [&](size_t x) {
        for (int j = 0; j < nn; j++) Sc[x * nn + j] = W((int)x, r2[j]);
    });
    f.irr = greedy_select(Sc, N1, nn, row);
    Sc.clear();
    Sc.shrink_to_fit();
    f.V.assign((size_t)row * N2, 0.f);
    for (int b = 0; b < row; b++)
        parallel_for(N2, [&](size_t j) { f.V[(size_t)b * N2 + j] = (float)W(f.irr[b], (int)j); });

    // 4: the middle matrix from np sampled points and wavenumbers
    const int np = std::min(mm, nn);
    const std::vector<int> r3 = draw_distinct(g, N1, np);
    const std::vector<int> r4 = draw_distinct(g, N2, np);
    std::vector<double> Us((size_t)np * col), Vs((size_t)row * np), Mes((size_t)np * np);
    for (int i = 0; i < np; i++)
        for (int a = 0; a < col; a++) Us[(size_t)i * col + a] = W(r3[i], f.jrr[a]);
    for (int b = 0; b < row; b++)
        for (int j = 0; j < np; j++) Vs[(size_t)b * np + j] = W(f.irr[b], r4[j]);
    for (int i = 0; i < np; i++)
        for (int j = 0; j < np; j++) Mes[(size_t)i * np + j] = W(r3[i], r4[j]);
    std::vector<double> Up, Vp;
    pinv(Us, np, col, 1e-8, Up);  // col x np
    pinv(Vs, row, np, 1e-8, Vp);  // np x row
    std::vector<double> T((size_t)col * np, 0.0);
    for (int a = 0; a < col; a++)
        for (int i = 0; i < np; i++) {
            const double u = Up[(size_t)a * np + i];
            if (u == 0.0) continue;
            for (int j = 0; j < np; j++) T[(size_t)a * np + j] += u * Mes[(size_t)i * np + j];
        }
    f.A.assign((size_t)col * row, 0.0);
    for (int a = 0; a < col; a++)
        for (int j = 0; j < np; j++) {
            const double t = T[(size_t)a * np + j];
            for (int b = 0; b < row; b++) f.A[(size_t)a * row + b] += t * Vp[(size_t)j * row + b];
        }
    f.nxx = nxx;
    f.nzz = nzz;
    f.row = row;
    f.col = col;
    return 0;
}

}  // namespace qp
