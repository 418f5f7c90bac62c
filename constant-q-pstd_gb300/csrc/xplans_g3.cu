// xplans_g3.cu -- x-pass kernels on the compiled long-line lengths of group 3
// (xplans_list.h, QP_XPLANS_G3).
#define QP_XGROUP 3
#define QP_XPLANS_GROUP QP_XPLANS_G3
#include "xplans.inc"
