// xplans_g2.cu -- x-pass kernels on the compiled convolution lengths of group 2
// (xplans_list.h, QP_XPLANS_G2).
#define QP_XGROUP 2
#define QP_XPLANS_GROUP QP_XPLANS_G2
#include "xplans.inc"
