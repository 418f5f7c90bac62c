// plain.h -- state of the plain (cuFFT) form of the step.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>

#include <string>

struct qpstd_shot;

namespace qp {

struct Wave;

struct PlainState {
    cufftHandle plan = 0;
    bool have_plan = false;
    float2* dis = nullptr;          // five complex nxx*nzz scratch fields (d_dis0..d_dis4)
    const float2 *HxM = nullptr, *HxP = nullptr, *HzM = nullptr, *HzP = nullptr;  // reference symbols
};

int plain_setup(qpstd_shot* s, std::string& err);
void plain_release(qpstd_shot* s);
// One reference-order step of w; returns 0, -1 (cuFFT error) or -2 (launch error).
int plain_step(qpstd_shot* s, Wave& w, float src, int t_filter, float eta, float* gather_row, const float* obs_row,
               bool ssg_on, bool image, long long* launches);

}  // namespace qp
