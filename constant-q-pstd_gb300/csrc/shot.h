// shot.h -- the device-resident state of one shot.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/qpstd.h"
#include "arena.h"
#include "plain.h"
#include "qpstd_internal.h"
#include "revolve.h"

namespace qp {

// One wavefield: 8 state fields (the reference's checkpoint set, in the order
// p, vx, vz, fipx, fipz, fivxx, fivzz, aux; storecheckpoints,
// sgpstd-qrtm/acsglw.cu:1946) followed by Dx, the x part of the next step's
// divergence that the fused schedule carries between passes.
struct Wave {
    float* st = nullptr;
    float* p(size_t N) { return st; }
    float* vx(size_t N) { return st + N; }
    float* vz(size_t N) { return st + 2 * N; }
    float* fipx(size_t N) { return st + 3 * N; }
    float* fipz(size_t N) { return st + 4 * N; }
    float* fivxx(size_t N) { return st + 5 * N; }
    float* fivzz(size_t N) { return st + 6 * N; }
    float* aux(size_t N) { return st + 7 * N; }
    float* Dx(size_t N) { return st + 8 * N; }
    // constant-Q: spectrum of the aux field produced at the end of a step;
    // aux_pending means the real aux field has not been refreshed from it yet
    float2* aux_spec = nullptr;
    bool aux_pending = false;
};

// Progress of one shot's revolve-driven RTM.
struct RtmRun {
    Revolve rv{1, 1};
    int ts = 0;
    bool first_sweep = true, first_rcv = true, done = false;
    int slice = 1 << 30;            // steps of an advance enqueued per action call
    int adv_t0 = 0, adv_t = 0, adv_left = 0;
};

}  // namespace qp

struct qpstd_shot;
int rtm_begin(qpstd_shot* s);
int rtm_action(qpstd_shot* s);  // 0: more actions, 1: finished, < 0: error code
// qpstd_shot_create with options: tune runs the lines-per-CTA autotuner, arena
// (may be null) supplies the device buffers.
int shot_create_ex(const qpstd_shot_desc* d, qpstd_shot** out, bool tune, qp::Arena* arena);
// Moves the shot to a new stream of CUDA priority prio (after its work so far).
int shot_set_priority(qpstd_shot* s, int prio);
// Modeling steps t0 .. t0+n-1 with the gather kept on the device (see shot.cu).
int model_slice(qpstd_shot* s, int t0, int n);
// A device buffer owned by the shot (its arena's when it has one); freed at destroy.
cudaError_t shot_malloc(qpstd_shot* s, void** p, size_t bytes);

struct qpstd_shot {
    qp::RtmRun run;
    qpstd_shot_desc d{};
    size_t N = 0;
    int nx = 0, nz = 0;
    bool visco = false, rtm = false;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    qp::Arena* arena = nullptr;  // device buffers come from here when set (server shots)
    qp::Wave src, rcv;
    float *div = nullptr, *Lz = nullptr;
    float *bbx = nullptr, *bbz = nullptr, *c1 = nullptr, *c2 = nullptr;
    const float *i_ax = nullptr, *i_bx = nullptr, *i_az = nullptr, *i_bz = nullptr;
    const float *h_ax = nullptr, *h_bx = nullptr, *h_az = nullptr, *h_bz = nullptr;
    const float *kx2 = nullptr, *kz2 = nullptr;
    const float2 *HxM = nullptr, *HxP = nullptr, *HzM = nullptr, *HzP = nullptr;
    qp::FFTPlanDev px{}, pz{};      // exact DFT plans (spectra of the constant-Q operators)
    qp::FFTPlanDev pxc{}, pzc{};    // convolution plans (separable operators)
    const float2 *cHxM = nullptr, *cHxP = nullptr, *cKx2 = nullptr;  // convolution multipliers
    const float2 *cHzM = nullptr, *cHzP = nullptr, *cKz2 = nullptr;
    int Lx = 1, Lzp = 1, ntile_x = 0;
    bool stage_x = false, stage_z = false;  // acoustic passes stage epilogue inputs
    int* rec_off = nullptr;
    qp::RecEntry* rec = nullptr;
    // constant-Q step
    int nzh = 0, Lzv = 1, Lxs = 1, Lxs3 = 1;
    int Lxs_exact = 1;                       // exact x-spectral pass (time-dependent filter) when xconv
    float2* spec[4] = {nullptr, nullptr, nullptr, nullptr};
    float* total = nullptr;
    float *y1 = nullptr, *y2 = nullptr, *y3c = nullptr, *y4c = nullptr;
    float *e1 = nullptr, *e2 = nullptr, *e3 = nullptr;
    float *kxsq = nullptr, *kzsq = nullptr;   // unnormalised squared wavenumbers
    // x-spectral passes with stationary symbols as per-kz convolutions (when
    // nxx needs Bluestein): tables nzh x pxc.m for (k^2)^(1/32), k^2,
    // (k^2)^(33/32), (k^2)^0.505
    bool xconv = false;
    const float* xtab[4] = {nullptr, nullptr, nullptr, nullptr};
    // Q-RTM filter: per eta, the last step at which it rounds to k^1.01 (see filter_is_ka)
    std::vector<std::pair<float, int>> ka_steps;
    // low-rank form of the pressure term (qpstd_shot_set_lowrank): row factors,
    // point weights c_b (row x N), per-kz convolution tables of the V_b
    // (row x nzh x (pxc.m/2+1)) and the row half spectra of one step
    int lr_row = 0, Llr = 1, Llrz = 1;
    float *lr_c = nullptr, *lr_tab = nullptr;
    float2* lr_Q = nullptr;
    int* rec_off_z = nullptr;                // receivers keyed by z-pass tile
    qp::RecEntry* rec_z = nullptr;
    // plain (cuFFT) form
    qp::PlainState plain;
    int plain_err = 0;
    std::vector<float> rik;
    float* gather = nullptr;
    float* store = nullptr;
    float* obs = nullptr;
    float *img = nullptr, *img_c = nullptr, *ssg = nullptr, *ssg_c = nullptr;
    long long launches = 0, fwd_steps = 0;
    // optional per-launch timing (CUDA events on the shot stream)
    bool pipe_first = true;
    bool prof = false;
    struct Timed { int kind; cudaEvent_t a, b; };
    std::vector<Timed> timed;
    std::vector<cudaEvent_t> evpool;
};
