// qpstd_internal.h -- structures shared by the host driver and the kernels.
#pragma once
#include <cuda_runtime.h>

#define QP_MAXST 10
// Threads per CTA of the pass kernels.  Kernels without a register cap below
// declare __launch_bounds__(QP_MAXTHREADS, 1), i.e. up to 80 registers.
#define QP_MAXTHREADS 768
// Register cap of the step's pass kernels: at 56 they compile spill-free and hold
// 4 (not 3) 256-thread line CTAs, or 9 (not 8) 128-thread ones, per SM (registers
// are allocated per warp in units of 256), which matters when many shots share
// the GPU.  The three-output x-spectral pass keeps
// 80: capped, it measured slower (at 56 without spills, four of its 54 KB CTAs per
// SM leave too little L1 for its table and twiddle loads).  The exact-DFT
// x-spectral pass (Bluestein transforms and the Q-RTM filter's exponentials)
// spills below 72 and takes that cap.
#define QP_PASS_REGS 56
// Passes whose plans use radices up to 12 run a 12-entry register array
// (fft_reg.cuh) and fit 48 registers spill-free (44 too, with the same 6 register
// units per warp): 10 (not 9) 128-thread CTAs per SM.
#define QP_R12_REGS 48
#define QP_WIDE_REGS 80
#define QP_EXACT_REGS 72
// Dynamic shared memory a pass kernel may request: the 227 KB per-CTA opt-in
// minus the static plan copies.
#define QP_SMEM_DYN_MAX (232448 - 1024)

namespace qp {

// One Stockham pass of a length-m transform.
struct FFTPass {
    int R;                 // radix (2..16)
    int ns;                // product of the radices of the earlier passes
    int B;                 // butterflies per line, m / R
    int twstride;          // m / (ns * R): stride into the length-m twiddle table
    unsigned ns_magic;     // ceil(2^32 / ns): j / ns = umulhi(j, ns_magic) for j < 2^16
};

// Device view of a line-FFT plan for one transform length n.
struct FFTPlanDev {
    int n;                 // logical length (the grid size along the line)
    int m;                 // inner transform length (n, or the Bluestein length)
    int blue;              // 1 if Bluestein is used
    int nst;               // number of passes of the length-m transform
    int tx;                // threads per line (>= max B, multiple of 32)
    FFTPass pass[QP_MAXST];
    const float2* w;       // m twiddles e^{-2 pi i k/m}
    const float2* chirp;   // n chirp values e^{-i pi k^2/n} (Bluestein)
    const float2* bhat;    // m values: DFT_m of the wrapped conj chirp, divided by m (Bluestein)
};

// Largest radix of a plan (host or device): kernels with plans up to radix 12
// can run the 12-entry register array.
__host__ __device__ inline int plan_max_radix(const FFTPlanDev& p) {
    int r = 0;
    for (int i = 0; i < p.nst; i++) r = (p.pass[i].R > r) ? p.pass[i].R : r;
    return r;
}

// Receiver / source bookkeeping for one x-tile of columns.
struct RecEntry {
    int gx, gz;   // padded-grid indices
    int ir;       // gather / obs column
    int inject;   // 1 if this entry is the winning index of its cell (Dirichlet side)
};

// ---------------------------------------------------------------------------
// z-line pass of the acoustic step (contiguous lines of length nzz).
//   do_v  : Pz = dz+ p; psi_pz; vz += dt bbz (Pz + psi_pz)
//   do_div: Dz = dz- vz; psi_vz; div = Dx + Dz + psi_vz; Lz = F^-1[kz^2 F div]
// ---------------------------------------------------------------------------
// The operators are applied as zero-padded circular convolutions on the
// length-m convolution plan pl; HzP, HzM, kz2 are their length-m multipliers.
struct AcZArgs {
    int nxx, nzz, L;
    FFTPlanDev pl;
    const float2 *HzP, *HzM;
    const float2* kz2;
    const float *h_az, *h_bz, *i_az, *i_bz;
    const float* bbz;
    float *p, *vz, *psi_pz, *psi_vz;
    const float* Dx;
    float *div, *Lz;
    float dt;
    int do_v, do_div;
    int stage;                    // stage epilogue inputs in shared memory (cp.async)
};

// ---------------------------------------------------------------------------
// x-line pass of the acoustic step (lines of length nxx, stride nzz); a CTA
// holds 2L consecutive z columns.
//   do_p : Lx = F^-1[kx^2 F div]; p += c1 (div - c2 (Lx + Lz)) (+ source,
//          receivers, illumination / imaging, Dirichlet injection)
//   do_v : Px = dx+ p; psi_px; vx += dt bbx (Px + psi_px)
//   do_dx: Dx = dx- vx + psi_vx (psi_vx updated)
// ---------------------------------------------------------------------------
// Fields the x pass stages in shared memory for its mode (bit f = field f):
// 0 div, 1 Lz, 2 p, 3 c1, 4 c2, 5 psi_px, 6 vx, 7 bbx, 8 psi_vx.  Each staged
// field takes nxx * 2L floats, in slot order (the rank of its bit).
__host__ __device__ inline unsigned xstage_fields(int do_p, int do_v, int do_dx) {
    unsigned m = 0;
    if (do_p) m |= 0x1Fu;
    if (do_v) m |= (1u << 2) | (1u << 5) | (1u << 6) | (1u << 7);
    if (do_dx) m |= (1u << 6) | (1u << 8);
    return m;
}
__host__ __device__ inline int xstage_count(unsigned m) {
    int n = 0;
    for (; m; m &= m - 1) n++;
    return n;
}

struct AcXArgs {
    int nxx, nzz, L, pml;
    FFTPlanDev pl;                // convolution plan along x
    const float2 *HxP, *HxM;      // length-m convolution multipliers
    const float2* kx2;
    const float *h_ax, *h_bx, *i_ax, *i_bx;
    const float *bbx, *c1, *c2;
    float *p, *vx, *psi_px, *psi_vx, *Dx;
    const float *div, *Lz;
    float dt;
    int do_p, do_v, do_dx;
    int xs, zs;
    float src;                    // amplitude added at (xs, zs) this step (0: none)
    const int* rec_off;           // per tile [ntile+1] offsets into rec
    const RecEntry* rec;
    float* gather_row;            // record p at receivers (NULL: off)
    const float* obs_row;         // Dirichlet injection values (NULL: off)
    float *ssg, *ssg_c;           // illumination accumulation, Kahan pair (NULL: off)
    float *img, *img_c;           // image accumulation, Kahan pair (NULL: off)
    const float* ps;              // source wavefield p for imaging
    int stage;                    // stage epilogue inputs in shared memory (cp.async)
};

// ---------------------------------------------------------------------------
// Constant-Q (vaps / qrtm) step.  The isotropic fractional symbols
// (k^2)^(1/32), k^2, (k^2)^(33/32), (k^2)^0.505 and the Q-RTM stabilised
// filter are not separable, so they run as 2-D transforms split into a z pass
// (real lines -> half spectra in kz, Hermitian packing of two real lines per
// complex line) and an x pass over the kz columns of those half spectra.
// Half spectra are stored x-major: S[ix*nzh + kz], nzh = nzz/2+1.
// ---------------------------------------------------------------------------

// z pass A: [aux <- z-inverse of the aux spectrum]; Dz, psi_vz, div = Dx+Dz;
// div -> half spectrum G.
struct VzArgsA {
    int nxx, nzz, nzh, L;
    FFTPlanDev pl;            // exact length-nzz DFT plan (spectra)
    FFTPlanDev plc;           // convolution plan for the z derivative
    const float2* HzM;        // convolution multiplier on plc
    const float *i_az, *i_bz;
    const float2* aux_spec;   // spectrum of the previous step's aux (null: aux already real)
    float* aux;
    float *vz, *psi_vz;
    const float* Dx;
    float* div;
    float2* G;
};

// x pass over half spectra: out_j = F_x^-1[ sym_j(kx,kz) F_x in ] / (nxx nzz).
//   mode 0: three outputs with (k^2)^(1/32), k^2, (k^2)^(33/32)
//   mode 1: one output with (k^2)^0.505
//   mode 2: one output with the Q-RTM stabilised symbol at time t_filter
struct VxsArgs {
    int nxx, nzz, nzh, L, mode;
    FFTPlanDev pl;            // exact length-nxx DFT plan (mode 2)
    FFTPlanDev plc;           // convolution plan along x (modes 0, 1)
    const float *kx2, *kz2;   // squared wavenumbers (unnormalised)
    const float2* in;
    float2 *out0, *out1, *out2;
    const float *tab0, *tab1, *tab2;  // per-kz convolution multipliers, nzh x (plc.m/2+1) (modes 0, 1)
    float norm;               // 1/(nxx*nzz)
    float eta6;               // eta * 1e-6 (mode 2)
    float tao, dt, tt;        // filter tau, dt, nt*dt (mode 2)
};

// Builds the per-kz convolution multipliers of a stationary 2-D symbol:
// for each kz, h = norm * IDFT_x(sym(kx, kz)) zero-padded and wrapped to
// plc.m, then out[kz*mh + k] = Re FFT_m(h)[k] / m for k = 0..m/2, mh = m/2+1
// (h is real and even, so the multipliers are real and even in k).
struct VtabArgs {
    int nxx, nzz, nzh, L, sym;  // sym: 0 (k^2)^(1/32), 1 k^2, 2 (k^2)^(33/32), 3 (k^2)^0.505,
                                //      4 the low-rank factor V (half grid, mirrored in kx)
    FFTPlanDev pl, plc;
    const float *kx2, *kz2;
    const float* V;             // sym 4: nxh x nzh values of one factor
    int nxh;
    float norm;
    float* out;
};

// Low-rank form of the constant-Q pressure term (qpstd_shot_set_lowrank):
// x-spectral pass: per kz column, Q_b = F_x^-1[Vt_b F_x G] / (nxx nzz) for the
// row factors b, as per-kz convolutions on the convolution plan (tables built
// from V by vz_convtab_kernel, sym 4).
struct LrxArgs {
    int nxx, nzh, L, row;
    FFTPlanDev plc;
    const float2* in;           // G, the z half spectrum of div
    float2* out;                // row half spectra, factor-major (b * nxx * nzh)
    const float* tab;           // row x nzh x (plc.m/2+1)
};
// z pass: psc(x) = sum_b c_b(x) Re F_z^-1[Q_b](x), c_b(x) = sum_a U[x][a] A[a][b].
struct LrsArgs {
    int nxx, nzz, nzh, L, row;
    FFTPlanDev pl;              // exact length-nzz plan
    const float2* Q;
    const float* c;             // row x nxx*nzz
    float* psc;
};

// z pass B: Y2, Y3, Y4 from their spectra; total; total -> half spectrum T.
struct VzArgsB {
    int nxx, nzz, nzh, L;
    FFTPlanDev pl;
    const float2 *Y2, *Y3, *Y4;
    const float* div;
    const float *y1, *y2, *y3c, *y4c;
    float* total;
    float2* T;
};

// z pass C: D from its spectrum; pressure update (+ source, receivers,
// illumination / imaging / injection); p -> half spectrum P; Pz, psi_pz, vz.
struct VzArgsC {
    int nxx, nzz, nzh, L, pml;
    FFTPlanDev pl;
    const float2* Dspec;      // null: no loss term (low-rank form: total = W{div}, e1 = rho vp^2 dt)
    const float* total;
    const float* aux;
    float* p;
    const float *e1, *e2, *e3;
    float sgn;                // -1 vaps (loss), +1 qrtm (compensation)
    int xs, zs;
    float src;
    const int* rec_off;       // receivers by z-pass tile (gx / (2L))
    const RecEntry* rec;
    float* gather_row;
    const float* obs_row;
    float *ssg, *ssg_c, *img, *img_c;
    const float* ps;
    float2* P;
    const float2* HzP;
    const float *h_az, *h_bz, *bbz;
    float *vz, *psi_pz;
    float dt;
};

// z pass that only turns a half spectrum back into a real field.
struct VzArgsI {
    int nxx, nzz, nzh, L;
    FFTPlanDev pl;
    const float2* spec;
    float* out;
};

}  // namespace qp
