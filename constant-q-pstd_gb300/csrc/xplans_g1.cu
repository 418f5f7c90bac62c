// xplans_g1.cu -- x-pass kernels on the compiled convolution lengths of group 1
// (xplans_list.h, QP_XPLANS_G1).
#define QP_XGROUP 1
#define QP_XPLANS_GROUP QP_XPLANS_G1
#include "xplans.inc"
