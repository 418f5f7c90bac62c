// xplans_list.h -- the convolution lengths compiled into the x passes.
//
// The separable x operators run as zero-padded circular convolutions on any
// smooth length m >= 2 nxx - 1 (host_setup.cpp, build_conv_plan_host), so the
// planner may round m up to one of these lengths, for which the x passes are
// compiled with the plan built in (CtFFT, fft_reg.cuh): straight-line passes of
// the exact radices, measured faster than the run-time plan.  Each entry lists
// the radices in the order the planner factors that length (odd radices first),
// so a compiled plan and the planner's plan for its length are the same passes.
// The lengths cover the windows of the batched Q-RTM workload (1319 <= m <=
// 4096) at steps of 7-15 %, the 439-wide window of the 160 x 398 model
// (900) and the 2461-wide one of the large RTM (5040).  Three groups, one
// translation unit each (xplans_g0.cu ..), keep the build parallel.
#pragma once

//
// Each entry is X(TX, radices...).  TX = 0: one butterfly per thread.  TX > 0
// (group 3, the long lines of wide windows, n about 3000 to 4600): TX threads
// per line, each running up to 16 / R butterflies of a radix-R pass, for
// lengths whose smallest radix would need more than 768 threads; only the x
// passes have them (the planner offers them for x lines alone).
#define QP_XPLANS_G0(X) X(0, 9, 10, 10) X(0, 12, 12, 10) X(0, 12, 12, 12) X(0, 14, 12, 12) X(0, 16, 14, 10)
#define QP_XPLANS_G1(X) X(0, 15, 14, 12) X(0, 15, 16, 12) X(0, 16, 16, 12) X(0, 15, 16, 14)
#define QP_XPLANS_G2(X) X(0, 16, 16, 14) X(0, 15, 16, 16) X(0, 16, 16, 16) X(0, 9, 7, 10, 8) X(0, 9, 10, 8, 8)
#define QP_XPLANS_G3(X) \
    X(512, 16, 16, 12, 2) X(768, 16, 16, 9, 3) X(512, 16, 16, 15, 2) X(512, 16, 16, 16, 2) X(768, 16, 16, 12, 3)
#define QP_XPLANS_ALL(X) QP_XPLANS_G0(X) QP_XPLANS_G1(X) QP_XPLANS_G2(X) QP_XPLANS_G3(X)
