// qpstd_internal.h -- structures shared by the host driver and the kernels.
#pragma once
#include <cuda_runtime.h>

#define QP_MAXST 24

namespace qp {

// Device view of a line-FFT plan for one transform length n.
struct FFTPlanDev {
    int n;                 // logical length (the grid size along the line)
    int m;                 // inner transform length (n, or the Bluestein length)
    int blue;              // 1 if Bluestein is used
    int nst;               // number of Stockham stages of the length-m transform
    int rad[QP_MAXST];     // radix of each stage
    const float2* w;       // m twiddles e^{-2 pi i k/m}
    const float2* chirp;   // n chirp values e^{-i pi k^2/n} (Bluestein)
    const float2* bhat;    // m values: DFT_m of the wrapped conj chirp, divided by m (Bluestein)
};

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
struct AcZArgs {
    int nxx, nzz, L;
    FFTPlanDev pl;
    const float2 *HzP, *HzM;
    const float* kz2;
    const float *h_az, *h_bz, *i_az, *i_bz;
    const float* bbz;
    float *p, *vz, *psi_pz, *psi_vz;
    const float* Dx;
    float *div, *Lz;
    float dt;
    int do_v, do_div;
};

// ---------------------------------------------------------------------------
// x-line pass of the acoustic step (lines of length nxx, stride nzz); a CTA
// holds 2L consecutive z columns.
//   do_p : Lx = F^-1[kx^2 F div]; p += c1 (div - c2 (Lx + Lz)) (+ source,
//          receivers, illumination / imaging, Dirichlet injection)
//   do_v : Px = dx+ p; psi_px; vx += dt bbx (Px + psi_px)
//   do_dx: Dx = dx- vx + psi_vx (psi_vx updated)
// ---------------------------------------------------------------------------
struct AcXArgs {
    int nxx, nzz, L, pml;
    FFTPlanDev pl;
    const float2 *HxP, *HxM;
    const float* kx2;
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
};

}  // namespace qp
