// ac_kernels.cu -- launchers of the acoustic pass kernels (ac_kernels.cuh).
#include "ac_kernels.cuh"
#include "xplans.cuh"

namespace qp {

size_t ac_zpass_smem(int L, int m, int nzz, bool stage) {
    return sizeof(float2) * (size_t)L * m + (stage ? sizeof(float) * 5 * (size_t)L * 2 * nzz : 0);
}
size_t ac_xpass_smem(int L, int m, int nxx, int nstaged) {
    return sizeof(float2) * (size_t)L * m + sizeof(float) * (size_t)nstaged * nxx * 2 * L;
}

// Plans compiled into the acoustic z pass (its convolution plan): 1728 = 12^3
// (nz 800 + CPML 30: 860 needs the convolution length), 660, 200 (see ZPlans
// in vz_kernels.cu).
using AcZPlans = PlanList<CtFFT<12, 12, 12>, CtFFT<11, 10, 6>, CtFFT<5, 5, 8>>;

void launch_ac_zpass(const AcZArgs& a, cudaStream_t s) {
    const int grid = (a.nxx + 2 * a.L - 1) / (2 * a.L);
    const size_t sm = ac_zpass_smem(a.L, a.pl.m, a.nzz, a.stage);
    const dim3 blk(a.pl.tx, a.L);
#define L_(FPT) ac_zpass_kernel<FPT><<<grid, blk, sm, s>>>(a)
    QP_DISPATCH(AcZPlans, a.pl, NoExtraPlan{}, plan_max_radix(a.pl) <= 12, L_);
#undef L_
}

void launch_ac_xpass(const AcXArgs& a, cudaStream_t s) {
    const int grid = (a.nzz + 2 * a.L - 1) / (2 * a.L);
    const int nst = a.stage ? xstage_count(xstage_fields(a.do_p, a.do_v, a.do_dx)) : 0;
    const size_t sm = ac_xpass_smem(a.L, a.pl.m, a.nxx, nst);
    // the instance without the p update carries only the transforms it runs
    const dim3 blk(a.pl.tx, a.L);
    if (xplan_launch_ac_xpass(a, s, dim3(grid), blk, sm)) return;  // a compiled length
    const bool r12 = plan_max_radix(a.pl) <= 12;
    if (a.do_p && r12) ac_xpass_kernel<true, RtFFT<12>><<<grid, blk, sm, s>>>(a);
    else if (a.do_p) ac_xpass_kernel<true, RtFFT<16>><<<grid, blk, sm, s>>>(a);
    else if (r12) ac_xpass_kernel<false, RtFFT<12>><<<grid, blk, sm, s>>>(a);
    else ac_xpass_kernel<false, RtFFT<16>><<<grid, blk, sm, s>>>(a);
}

int ac_set_smem_limits() {
    const int lim = QP_SMEM_DYN_MAX;
    int bad = 0;
    auto z = [&](auto fp) {
        bad |= cudaFuncSetAttribute(ac_zpass_kernel<decltype(fp)>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
               cudaSuccess;
    };
    z(RtFFT<12>{});
    z(RtFFT<16>{});
    for_each_plan(AcZPlans{}, z);
    auto x = [&](auto fp) {
        using F = decltype(fp);
        bad |= cudaFuncSetAttribute(ac_xpass_kernel<true, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
               cudaSuccess;
        bad |= cudaFuncSetAttribute(ac_xpass_kernel<false, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
               cudaSuccess;
    };
    x(RtFFT<12>{});
    x(RtFFT<16>{});
    bad |= xplan_set_all_limits(lim, 200 * 1024);
    return bad ? -1 : 0;
}

}  // namespace qp
