// xplans.cuh -- launchers of the x-pass kernels on the compiled convolution
// lengths (xplans_list.h); each group is instantiated in its own translation
// unit (xplans_g0.cu ...).
#pragma once
#include <cuda_runtime.h>

#include "qpstd_internal.h"

namespace qp {

// Per group G (xplans_g<G>.cu): launch the kernel on plan a.pl / a.plc when it
// is one of the group's compiled lengths and return true; else launch nothing
// and return false.  set_limits: cudaFuncSetAttribute (dynamic shared memory)
// for every instance of the group.
// The exact x-spectral pass, the table builder and the low-rank x pass have
// compiled instances for the long plans (TX > 0) only; shorter lengths run them
// on the run-time plan.
#define QP_XPLAN_DECLARE(G)                                                                            \
    bool xplan_ac_xpass_g##G(const AcXArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem);   \
    bool xplan_xspec_conv_g##G(const VxsArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem); \
    bool xplan_xspec_g##G(const VxsArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem);      \
    bool xplan_convtab_g##G(const VtabArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem);   \
    bool xplan_lr_xconv_g##G(const LrxArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem);   \
    int xplan_set_limits_g##G(int ac_limit, int vz_limit);
QP_XPLAN_DECLARE(0)
QP_XPLAN_DECLARE(1)
QP_XPLAN_DECLARE(2)
QP_XPLAN_DECLARE(3)

#define QP_XPLAN_ANY(F, ...) (F##_g0(__VA_ARGS__) || F##_g1(__VA_ARGS__) || F##_g2(__VA_ARGS__) || F##_g3(__VA_ARGS__))
inline bool xplan_launch_ac_xpass(const AcXArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem) {
    return QP_XPLAN_ANY(xplan_ac_xpass, a, s, grid, blk, smem);
}
inline bool xplan_launch_xspec_conv(const VxsArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem) {
    return QP_XPLAN_ANY(xplan_xspec_conv, a, s, grid, blk, smem);
}
inline bool xplan_launch_xspec(const VxsArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem) {
    return QP_XPLAN_ANY(xplan_xspec, a, s, grid, blk, smem);
}
inline bool xplan_launch_convtab(const VtabArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem) {
    return QP_XPLAN_ANY(xplan_convtab, a, s, grid, blk, smem);
}
inline bool xplan_launch_lr_xconv(const LrxArgs& a, cudaStream_t s, dim3 grid, dim3 blk, size_t smem) {
    return QP_XPLAN_ANY(xplan_lr_xconv, a, s, grid, blk, smem);
}
inline int xplan_set_all_limits(int ac_limit, int vz_limit) {
    return xplan_set_limits_g0(ac_limit, vz_limit) | xplan_set_limits_g1(ac_limit, vz_limit) |
           xplan_set_limits_g2(ac_limit, vz_limit) | xplan_set_limits_g3(ac_limit, vz_limit);
}

}  // namespace qp
