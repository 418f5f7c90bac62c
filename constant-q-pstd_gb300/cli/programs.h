// programs.h -- host side of the four programs (aps, vaps, artm, qrtm) and of
// the geometry generator, for the native command-line tool over libqpstd.
//
// The reference builds each program from an MPI main (parameter file, shot
// distribution, model and geometry files, coefficient setup) and one CUDA file
// with acforward.  The tool reads the same parameter files and writes the same
// output files; the shots of a process run through the C ABI (the shot server
// by default, so several shots share the GPU).
#pragma once
#include <string>
#include <vector>

namespace qpcli {

enum Program { APS = 0, VAPS = 1, ARTM = 2, QRTM = 3 };

// What a program's parameter file holds (the reference's input_ac2d_parameters
// of each program; absent fields keep their defaults).
struct Params {
    int shotnum = 0, tmax = 0, nxt = 0, nzt = 0;
    float dt = 0.f;          // milliseconds, as in the file
    float fd = 0.f, fo = 0.f, dx = 0.f, dz = 0.f, disx = 0.f;
    float v0 = 0.f, etas = 0.f, etar = 0.f;
    std::string trace, shotx, shotz, gxp, gzp, vp, rho, qp, rec;
    int flagout = 0, flagsource = 2, snapnum = 0;
};

// Default parameter file of each program, relative to its working directory
// (sgpstd-qmodeling/funca.c:18, func.c:18; sgpstd-qrtm/funca.c:20, func.c:20).
const char *default_params(Program p);
const char *program_name(Program p);

// One value of a parameter file, in file order: its kind (I int, F float,
// S string) and the member of Params it fills.
enum FieldKind { FIELD_INT, FIELD_FLOAT, FIELD_STRING };
struct Field {
    FieldKind k;
    void *p;
    const char *what;
};
std::vector<Field> param_layout(Program p, Params &o);

// Reads a parameter file laid out as the program's reader expects: every value
// follows one label line.  Returns false with a message on a short or
// malformed file.
bool read_params(Program p, const std::string &path, Params &out, std::string &err);

// geometry/parameters.txt (geometry/geometry2d.c:27-84)
struct GeometryParams {
    int shotnum = 0;
    float sx0 = 0.f, sxdx = 0.f, sdep = 0.f, rdep = 0.f, offset = 0.f, trdx = 0.f, dx = 0.f, dz = 0.f;
    int nx = 0, nz = 0;
};
bool read_geometry_params(const std::string &path, GeometryParams &g, std::string &err);

// Split-spread geometry files in dir: tracenum.bin (int32 per shot),
// shotxp.bin, shotzp.bin, gxp<i>.bin, gzp<i>.bin (float32), as
// geometry/geometry2d.c:87-149 writes them.  Returns false with a message when
// a shot or receiver falls outside the model.
bool write_geometry(const GeometryParams &g, const std::string &dir, std::string &err, bool verbose);

// Setup on the full model, in the reference's float arithmetic.
void cal_bbx_bbz(int nx, int nz, const float *rho, float *bbx, float *bbz);                 // func.c:205
void rik_cal(int tmax, float dt, float fd, int flag, float *rik);                           // func.c:237
void transfermodel(int n, float fd, float fo, const float *vp, const float *qp, float *gam, float *lam,
                   float *vwd, float *tao);                                                 // func.c:939
void get_max_min(int n, const float *a, float *vmax, float *vmin);                          // func.c:555
float cfl_number(float vmax, float dt, float dx, float dz);                                 // func.c:569

// Shots of process `rank` among `nranks` (one GPU each): the first shot id and
// the count (acousticsgps4.c:254-270 with GPU_N = 1).
void distribute(int shotnum, int nranks, int rank, int *first, int *count);

// Window extent shared by a process's shots: the largest source-receiver
// offset over its shots (acousticsgps4.c:304-330), and the window width
// nx = (int)(2 (sroffmx + disx) / dx + 1.5) (:333-335).
int window_width(float sroffmx, float disx, float dx);

}  // namespace qpcli
