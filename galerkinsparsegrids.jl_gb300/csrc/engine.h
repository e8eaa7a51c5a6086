// engine.h -- device-side data structures shared by the kernels and the host
// drivers of libsgdg.  Plain C structs: they are copied to device memory as-is.
#pragma once
#include <cstddef>
#include <cstdint>

namespace sgdg {

// ---- plain form: FP64 CSR ---------------------------------------------------
// Rows longer than `split` entries are summed in segments of `split` by one
// warp each (partial sums in `partial`), then combined per row in segment
// order -- so a handful of very long rows (a coarse mode touched by every
// coefficient) does not serialise the launch, and results stay deterministic.
constexpr int kCsrBins = 6;    // row bins of the CSR kernels: 1, 2, 4, ..., 32 lanes per row
constexpr int kCsrMaxVec = 4;  // vectors one pass of the multi-vector SpMV carries

struct DevCSR {
    int64_t m;
    int64_t nnz;
    const int64_t* rowptr;
    const int32_t* col;
    const double* val;
    // rows of at most `split` entries by bin, ascending within a bin: bin b
    // (2^b lanes per row) holds bin_rows[bin_first[b] .. bin_first[b + 1])
    // and is served by grid blocks bin_block[b] .. bin_block[b + 1]
    const int32_t* bin_rows;
    int64_t bin_first[kCsrBins + 1];
    int bin_block[kCsrBins + 1];
    int64_t split;            // longest row a single row group sums
    int64_t nlong, nseg;      // rows longer than split, their segments
    const int32_t* long_row;  // nlong: the rows
    const int32_t* long_seg;  // nlong + 1: first segment of each long row
    const int64_t* seg_begin; // segment s is [seg_begin[s], seg_end[s])
    const int64_t* seg_end;
    double* partial;          // kCsrMaxVec * nseg: segment sums, one block of nseg per vector
};

// ---- chosen form: matrix-free FP32 pencil apply, FP64 RK state --------------
//
// Solves with equal (D, k, n, scheme, kind) form a class.  A class keeps its
// solves' vectors in arenas (slot-major: slot s owns [s*Ns, (s+1)*Ns)), so a
// tile may take columns from several solves.  One launch per RK4 step runs an
// ordered work list: for every group of slots and every stage, one pass per
// dimension (pencil tiles: sweep the 1D operator, accumulate into rhs); the
// last pass applies the RK stage update to the elements it completes.  Each
// phase waits for the previous phase of its group, and a stage's gathers wait
// for the group's RK update of the stage before.
enum : int { MF_KIND_ADVECT = 0, MF_KIND_WAVE = 1, MF_KIND_VLASOV = 2 };
// TILE_RK: the pass completes the right-hand side and applies the RK4 update;
// TILE_STORE: the result goes to a scratch vector; TILE_WACC: times a point
// weight, added into the point-basis accumulator; TILE_WAIT_IN: the input
// was written by the previous phase of this launch (wait before gathering);
// TILE_SUMIN: the input is the sum of the D scratch vectors src, src + 2, ...
// (the per-dimension point products of the Vlasov right-hand side), added in
// that order.
enum : int {
    TILE_FIRST = 1, TILE_LAST = 2, TILE_RK = 4, TILE_STORE = 8, TILE_WACC = 16, TILE_WAIT_IN = 32, TILE_SUMIN = 64
};
// MFItem::tab; 0..3: the nodal transforms.  TABLE_SQUARE: the wave's
// D_d D_d on the pencil's line as one sweep of the squared line operator
// (otherwise the wave sweeps the derivative table twice).
enum : int { TABLE_DERIVATIVE = -1, TABLE_SQUARE = -2 };
constexpr int kMFMaxLevels = 16;  // n + 1 <= 16 line lengths per class

struct MFClass {
    const int32_t* s_rowptr;  // 1D operator, block CSR over 2^n row blocks (2^n + 1 entries)
    const int32_t* s_ent;     // per stored block: column block << 12 | distinct block id
    const float* s_val;       // distinct blocks: k rows of (hi, lo) pairs, each row padded to rs floats
    // the squared line operators (wave): one block-CSR table per line length
    // lm = 1..n+1 (its 2^(lm-1) + 1 row pointers at q_rowptr + q_roff[lm - 1],
    // indexing q_ent); the distinct blocks are shared by all line lengths
    const int32_t* q_rowptr;
    const int32_t* q_ent;
    const float* q_val;
    int32_t q_roff[kMFMaxLevels];
    const int64_t* blockoff;  // level-block offsets of every pencil of the class
    double* y;                // arenas, nslots * Ns
    double* acc;
    // FP32 stage inputs: stage s of a step reads u[(s - 1) % 4] and its RK
    // update writes u[s % 4] (the fourth stage u[0], the next step's input),
    // so within a whole-step launch no buffer is written after it was read
    float* u[4];
    float* rhs;               // nslots * N
    const double* dt;         // per slot: dt, dt / 2, dt / 6
    const float* coef;        // per slot, 16 entries: factor on D_d as hi[8], lo[8]
    const int32_t* status;    // per slot, nonzero = skip the RK update
    int32_t N, Ns;
    int32_t nslots;           // slots of the arenas
    int32_t D, k, kD, kind, rs;
    int32_t s_nrow, s_nent, s_nval;  // table sizes (ints, ints, floats) for the shared-memory copy
    int32_t s_shared;                // 1: pass tiles read a shared-memory copy of the table; 0: global memory
    // Vlasov classes: the four nodal transforms (1D block tables, read through
    // L1), scratch vectors and the point weights of the D point products
    int32_t t_nrow[4], t_nent[4], t_nval[4];  // their sizes, as s_nrow, s_nent, s_nval
    const int32_t* t_rowptr[4];
    const int32_t* t_ent[4];
    const float* t_val[4];
    float* vbase;             // scratch vector v of slot s at vbase + v vstride + s N (2 per phase dimension)
    int64_t vstride;
    const float* vw;          // per slot 2 x D x N: weight of term d at [d N] (hi) and [(D + d) N] (lo)
};

// bytes of the shared-memory copy of a class's 1D operator table
#ifdef __CUDACC__
__host__ __device__
#endif
inline int mf_table_bytes(int nrow, int nent, int nval) {
    return (((nrow + nent) * 4 + 15) / 16) * 16 + nval * 4;
}
// tables above this size are read from global memory (their row lists grow
// like 2^n n; the distinct blocks stay a few hundred)
constexpr int kMFTableSmemMax = 48 * 1024;

struct MFItem {
    int16_t tab;       // 1D table: TABLE_DERIVATIVE or a nodal transform 0..3
    int16_t cls;
    int16_t d;         // 0-based dimension of the pencils
    int16_t flags;     // TILE_*
    int16_t src;       // input: -1 the stage input, 0..2 a scratch vector
    int16_t dst;       // TILE_STORE / TILE_WACC output vector
    int16_t wsel;      // TILE_WACC: the weight (term) index
    int16_t stage;     // RK stage 1..4 of the item in a whole-step list; 0: the launch's stage
    int32_t wait_ctr;  // counter to wait for (-1: none) ...
    int32_t wait_need; // ... until it reaches this value
    int32_t win_ctr;   // whole-step list: counter of the RK phase that wrote the stage input (<= 0: none) ...
    int32_t win_need;  // ... which must reach this value before the input is gathered
    int32_t done_ctr;  // counter incremented when the item is done
    int32_t lmax;      // pass: 1-based max level of the pencil along d
    int32_t lp;        // pass: log2 prod_{q<d} cells_q
    int32_t boff;      // pass: first level-block offset of the pencil in blockoff
    int32_t R;         // pass: columns per solve
    int32_t g0;        // pass: first class column (slot*R + r)
    int32_t W;         // pass: columns (multiple of the per-thread column count)
    int32_t Wv;        // pass: valid columns
    int32_t kd1;       // pass: k^d
    int32_t kDm1;      // pass: k^(D-1)
    int32_t rlong;     // pass: leading row blocks swept by a whole warp each
    uint32_t rmagic;   // pass: g / R = (g * rmagic) >> rshift for 0 <= g < 2^31 (mf_divisor)
    int32_t rshift;
};

// (magic, shift) of the division by an invariant d >= 1 for numerators below
// 2^31: Granlund and Montgomery (PLDI 1994), Theorem 4.2 with N = 31,
// l = ceil(log2 d), magic = floor(2^(31+l) / d) + 1 (< 2^32), shift = 31 + l.
inline void mf_divisor(int32_t d, uint32_t* magic, int32_t* shift) {
    int l = 0;
    while ((1LL << l) < (long long)d) l++;
    *magic = (uint32_t)(((1ULL << (31 + l)) / (unsigned long long)d) + 1ULL);
    *shift = 31 + l;
}

constexpr int kMFThreads = 256;  // 8 warps share one copy of the operator table
constexpr int kMFThreadsLog2 = 8;
static_assert(1 << kMFThreadsLog2 == kMFThreads, "kMFThreadsLog2");
constexpr int kSpinLimit = 1 << 22;  // polls of a dependency counter before giving up

// Tile shape of the pass tiles of one (D, k), chosen by the autotuner:
// a tile has cpt * max(1, kMFThreads / nrb) * 2^wlog columns (at least cpt; nrb =
// row blocks of the pencil), and the row blocks of levels <= lmax - coop are
// warp-cooperative.  Narrower tiles need less shared memory (more CTAs per
// SM), wider ones amortise each item's fixed cost.
struct MFTile {
    int wlog = 0;
    int coop = 4;
};
constexpr int kMFWlogMin = -2, kMFWlogMax = 3;
MFTile mf_tile(int D, int k);                 // tuned shape, or the default
bool mf_tile_tuned(int D, int k);
void mf_set_tile(int D, int k, const MFTile& t);
void mf_clear_tiles();

inline int mf_rlong(int lmax, int coop) { return lmax > coop ? 1 << (lmax - 1 - coop) : 0; }
// bytes of dynamic shared memory a pass tile of W columns over nrb row blocks needs
// (three int tables per column, an int2 per row padded to an even row count,
// the tile and its sweep output)
inline size_t mf_tile_smem(int k, int nrb, int W) {
    const size_t m = (size_t)k * nrb;
    return 4 * (3 * (size_t)W + 2 * ((m + 1) & ~(size_t)1) + m * W * 2);
}
constexpr size_t kMFTileSmemMax = 64 * 1024;  // wider tiles are narrowed to fit
// columns of a pass tile (a power of two)
inline int mf_tile_cols(int k, int cpt, int nrb, int wlog) {
    int W = cpt * (nrb < kMFThreads ? kMFThreads / nrb : 1);
    W = wlog >= 0 ? W << wlog : W >> -wlog;
    if (W < cpt) W = cpt;
    while (W > cpt && mf_tile_smem(k, nrb, W) > kMFTileSmemMax) W >>= 1;
    return W;
}

}  // namespace sgdg
