// lowrank.h -- low-rank form of the mixed-domain constant-Q symbol.
#pragma once
#include <cstdint>
#include <vector>

#include "qpstd_internal.h"

namespace qp {

// W(x, k) = sinc(vp dt k^(1+g) / 2) k^g sqrt(1 + dt tau k^1.01 / 2), sinc(u) = sin(u)/u
// (sgpstd-qmodeling/sglowrank.c:251-257, 301, 339, 398).
double lowrank_symbol(double vp, double gam, double tao, double dt, double k);

// |k| on the half grid (nxh = nxx/2+1) x (nzh = nzz/2+1), k[0] = 1e-6
// (cal_k2dh, sgpstd-qmodeling/func.c:783-811).
void lowrank_khalf(int nxx, int nzz, double dx, double dz, std::vector<double>& k);

// The decomposition W(x_i, k_j) ~ sum_a sum_b U[i][a] A[a][b] V[b][j]
// (acsglowrank2d, sgpstd-qmodeling/sglowrank.c:148-480), in FP64:
//   U: N1 x col (columns of W at the selected wavenumbers jrr),
//   V: row x N2 (rows of W at the selected points irr),
//   A: col x row = pinv(Us) Mes pinv(Vs) on np random points and wavenumbers.
struct LowRankFactors {
    int nxx = 0, nzz = 0, row = 0, col = 0;
    std::vector<float> U, V;
    std::vector<double> A;
    std::vector<int> jrr, irr;
};
int lowrank_decompose(int nxx, int nzz, double dx, double dz, double dt, const float* vp, const float* tao,
                      const float* gam, int row, int col, uint64_t seed, LowRankFactors& f);

// Moore-Penrose inverse of the m x n row-major matrix M (n x m result);
// singular values at or below eps * sigma_max are treated as zero.
void pinv(const std::vector<double>& M, int m, int n, double eps, std::vector<double>& P);

// ---- device apply: out = sum_b c_b(x) Re F^-1[Vt_b(k) F in](x) / N -------------
// c_b(x) = sum_a U[x][a] A[a][b]; Vt_b is V_b mirrored to the full k grid.
struct LrZArgs {
    int nxx, nzz, nzh, L, row;
    FFTPlanDev pl;               // exact length-nzz plan
    const float* in;             // zfwd: real field
    float2* spec;                // zfwd: half spectrum out; zinv: row half spectra in
    const float* c;              // zinv: row x N1 point weights
    float* out;                  // zinv: real field
};
struct LrXArgs {
    int nxx, nzz, nzh, nxh, L, row;
    FFTPlanDev pl;               // exact length-nxx plan
    const float* V;              // row x (nxh*nzh)
    const float2* in;            // half spectrum (z transformed)
    float2* out;                 // row half spectra
    float norm;                  // 1/(nxx*nzz)
};
void launch_lr_zfwd(const LrZArgs& a, cudaStream_t s);
void launch_lr_xspec(const LrXArgs& a, cudaStream_t s);
void launch_lr_zinv(const LrZArgs& a, cudaStream_t s);
int lr_set_smem_limits();

}  // namespace qp
