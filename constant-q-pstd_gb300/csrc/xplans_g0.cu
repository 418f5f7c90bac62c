// xplans_g0.cu -- x-pass kernels on the compiled convolution lengths of group 0
// (xplans_list.h, QP_XPLANS_G0).
#define QP_XGROUP 0
#define QP_XPLANS_GROUP QP_XPLANS_G0
#include "xplans.inc"
