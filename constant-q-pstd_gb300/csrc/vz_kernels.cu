// vz_kernels.cu -- launchers of the constant-Q pass kernels (vz_kernels.cuh).
#include "vz_kernels.cuh"
#include "xplans.cuh"

namespace qp {

// ---- launchers -------------------------------------------------------------------
static size_t lsm(int L, int m, int nbuf) { return sizeof(float2) * (size_t)nbuf * L * m; }
static int zgrid(int nxx, int L) { return (nxx + 2 * L - 1) / (2 * L); }

// Plans compiled into the z passes (CtFFT): 660 = 11*10*6 (the Q-RTM batch's
// nz 600 + CPML 30), 200 = 5*5*8 (nz 160 + CPML 20).  Other lengths run the
// run-time plan (RtFFT, 12- or 16-entry register array).
using ZPlans = PlanList<CtFFT<11, 10, 6>, CtFFT<5, 5, 8>>;


void launch_vz_passA(const VzArgsA& a, cudaStream_t s) {
    const dim3 blk(max(a.pl.tx, a.plc.tx), a.L);
    const size_t sm = lsm(a.L, max(a.pl.m, a.plc.m), 1);
    const bool r12 = plan_max_radix(a.pl) <= 12 && plan_max_radix(a.plc) <= 12;
    auto same_plc = [&](auto fp) { return decltype(fp)::matches(a.plc); };
#define L_(FPT) vz_passA_kernel<FPT><<<zgrid(a.nxx, a.L), blk, sm, s>>>(a)
    QP_DISPATCH(ZPlans, a.pl, same_plc, r12, L_);
#undef L_
}
void launch_vz_xspec(const VxsArgs& a, cudaStream_t s) {
    const int grid = (a.nzh + a.L - 1) / a.L;
    const size_t sm = lsm(a.L, a.pl.m, a.mode == 0 ? 2 : 1);
    if (xplan_launch_xspec(a, s, dim3(grid), dim3(a.pl.tx, a.L), sm)) return;  // a compiled long plan
    if (plan_max_radix(a.pl) <= 12) vz_xspec_kernel<RtFFT<12>><<<grid, dim3(a.pl.tx, a.L), sm, s>>>(a);
    else vz_xspec_kernel<RtFFT<16>><<<grid, dim3(a.pl.tx, a.L), sm, s>>>(a);
}
void launch_vz_xspec_conv(const VxsArgs& a, cudaStream_t s) {
    const int grid = (a.nzh + a.L - 1) / a.L;
    const dim3 blk(a.plc.tx, a.L);
    if (xplan_launch_xspec_conv(a, s, dim3(grid), blk, lsm(a.L, a.plc.m, a.mode == 0 ? 2 : 1))) return;
    const bool r12 = plan_max_radix(a.plc) <= 12;
    if (a.mode == 0 && r12) vz_xspec_conv_kernel<3, RtFFT<12>><<<grid, blk, lsm(a.L, a.plc.m, 2), s>>>(a);
    else if (a.mode == 0) vz_xspec_conv_kernel<3, RtFFT<16>><<<grid, blk, lsm(a.L, a.plc.m, 2), s>>>(a);
    else if (r12) vz_xspec_conv_kernel<1, RtFFT<12>><<<grid, blk, lsm(a.L, a.plc.m, 1), s>>>(a);
    else vz_xspec_conv_kernel<1, RtFFT<16>><<<grid, blk, lsm(a.L, a.plc.m, 1), s>>>(a);
}
void launch_vz_convtab(const VtabArgs& a, cudaStream_t s) {
    const int grid = (a.nzh + a.L - 1) / a.L;
    const dim3 blk(max(a.pl.tx, a.plc.tx), a.L);
    const size_t sm = lsm(a.L, max(a.pl.m, a.plc.m), 1);
    if (xplan_launch_convtab(a, s, dim3(grid), blk, sm)) return;  // a compiled long plan
    vz_convtab_kernel<RtFFT<16>><<<grid, blk, sm, s>>>(a);
}
void launch_lr_xconv(const LrxArgs& a, cudaStream_t s) {
    const int grid = (a.nzh + a.L - 1) / a.L;
    const dim3 blk(a.plc.tx, a.L);
    const size_t sm = lsm(a.L, a.plc.m, 2);
    if (xplan_launch_lr_xconv(a, s, dim3(grid), blk, sm)) return;  // a compiled long plan
    if (plan_max_radix(a.plc) <= 12) lr_xconv_kernel<RtFFT<12>><<<grid, blk, sm, s>>>(a);
    else lr_xconv_kernel<RtFFT<16>><<<grid, blk, sm, s>>>(a);
}
void launch_lr_zsum(const LrsArgs& a, cudaStream_t s) {
    const dim3 blk(a.pl.tx, a.L);
    const size_t sm = lsm(a.L, a.pl.m, 2);
#define L_(FPT)                                                                         \
    for (int b0 = 0; b0 < a.row; b0 += lr_terms<FPT>())                                 \
    lr_zsum_kernel<FPT><<<zgrid(a.nxx, a.L), blk, sm, s>>>(a, b0, min(lr_terms<FPT>(), a.row - b0))
    QP_DISPATCH(ZPlans, a.pl, NoExtraPlan{}, plan_max_radix(a.pl) <= 12, L_);
#undef L_
}

void launch_vz_passB(const VzArgsB& a, cudaStream_t s) {
    const dim3 blk(a.pl.tx, a.L);
    const size_t sm = lsm(a.L, a.pl.m, 2);
#define L_(FPT) vz_passB_kernel<FPT><<<zgrid(a.nxx, a.L), blk, sm, s>>>(a)
    QP_DISPATCH(ZPlans, a.pl, NoExtraPlan{}, plan_max_radix(a.pl) <= 12, L_);
#undef L_
}
void launch_vz_passC(const VzArgsC& a, cudaStream_t s) {
    const dim3 blk(a.pl.tx, a.L);
    const size_t sm = lsm(a.L, a.pl.m, 1);
#define L_(FPT) vz_passC_kernel<FPT><<<zgrid(a.nxx, a.L), blk, sm, s>>>(a)
    QP_DISPATCH(ZPlans, a.pl, NoExtraPlan{}, plan_max_radix(a.pl) <= 12, L_);
#undef L_
}
void launch_vz_zinv(const VzArgsI& a, cudaStream_t s) {
    const dim3 blk(a.pl.tx, a.L);
    const size_t sm = lsm(a.L, a.pl.m, 1);
#define L_(FPT) vz_zinv_kernel<FPT><<<zgrid(a.nxx, a.L), blk, sm, s>>>(a)
    QP_DISPATCH(ZPlans, a.pl, NoExtraPlan{}, plan_max_radix(a.pl) <= 12, L_);
#undef L_
}

template <class FP> static int vz_set_limits_one() {
    const int lim = 200 * 1024;
    int bad = 0;
    bad |= cudaFuncSetAttribute(vz_passA_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_passB_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_passC_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_zinv_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(lr_zsum_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    return bad;
}

int vz_set_smem_limits() {
    const int lim = 200 * 1024;
    int bad = vz_set_limits_one<RtFFT<12>>() | vz_set_limits_one<RtFFT<16>>();
    for_each_plan(ZPlans{}, [&](auto fp) { bad |= vz_set_limits_one<decltype(fp)>(); });
    bad |= cudaFuncSetAttribute(vz_xspec_kernel<RtFFT<12>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_kernel<RtFFT<16>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_conv_kernel<3, RtFFT<12>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_conv_kernel<3, RtFFT<16>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_conv_kernel<1, RtFFT<12>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_xspec_conv_kernel<1, RtFFT<16>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(vz_convtab_kernel<RtFFT<16>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(lr_xconv_kernel<RtFFT<12>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    bad |= cudaFuncSetAttribute(lr_xconv_kernel<RtFFT<16>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess;
    return bad ? -1 : 0;
}

}  // namespace qp
