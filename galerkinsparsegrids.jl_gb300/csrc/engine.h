// engine.h -- device-side data structures shared by the kernels and the host
// drivers of libsgdg.  Plain C structs: they are copied to device memory as-is.
#pragma once
#include <cstdint>

namespace sgdg {

// ---- plain form: FP64 CSR ---------------------------------------------------
struct DevCSR {
    int64_t m;
    int64_t nnz;
    const int64_t* rowptr;
    const int32_t* col;
    const double* val;
    int vs;  // lanes per row
};

// ---- chosen form: matrix-free FP32 pencil apply, FP64 RK state --------------
enum : int { MF_KIND_ADVECT = 0, MF_KIND_WAVE = 1 };
enum : int { TILE_FIRST = 1, TILE_LAST = 2 };

struct MFSolve {
    double* y;       // RK state (N or 2N for the wave)
    double* acc;     // RK accumulator
    float* u[2];     // stage inputs/outputs (ping-pong), same length as y
    float* rhs;      // partial sum over dimensions, N
    const int32_t* s_rowptr;  // 1D operator, block CSR over 2^n row blocks
    const int32_t* s_colblk;
    const float* s_val;       // blocks of kk floats, [i][j] row-major
    const int64_t* blockoff;  // pencil level-block offsets (all pencils of this solve)
    double dt;
    int64_t N;       // operator size (coefficients per field)
    int D, k, kk, kind;
    int kD;          // k^D
    int status;      // nonzero once the solve is stopped (cancel / error)
    float coef[8];   // factor on D_d (advection: -a_d; wave: 1)
};

struct MFTile {
    int32_t solve;
    int16_t d;       // 0-based dimension
    int16_t flags;   // TILE_FIRST | TILE_LAST
    int32_t lmax;    // 1-based max level of the pencil along d
    int32_t lp;      // log2 prod_{q<d} cells_q
    int32_t boff;    // index of the pencil's first level-block offset in blockoff
    int32_t r0;      // first column of the chunk
    int32_t wc;      // columns in the chunk
    int32_t kd1;     // k^d (stride of dimension d's mode)
    int32_t kDm1;    // k^(D-1)
};

constexpr int kMFThreads = 256;

}  // namespace sgdg
