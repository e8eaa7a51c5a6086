// sgdg_core.h -- internal host-side structures of libsgdg (not part of the C ABI).
//
// Naming follows GalerkinSparseGrids.jl: levels are 1-based like the reference's
// CartesianIndex levels (level L means hierarchical level L-1), cells and modes
// are 1-based in the public index map and 0-based inside the library.
#pragma once
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sgdg {

constexpr int kKMax = 10;  // K_max, src/1d_dg_functions.jl:7
constexpr int kDMax = 8;   // largest dimension the library indexes

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------- basis ----
// Hierarchical multiwavelet basis on [-1,1] (src/dg_basis.jl:185-190) and the
// normalised Legendre polynomials (src/dg_basis.jl:88-94).  A basis function
// is stored as 2k coefficients: x^i for i<k and sgn(x) x^i for i>=k.
struct Basis1D {
    int k = 0;
    std::vector<double> dg;   // dg[mode*2k + coef]
    std::vector<double> leg;  // leg[m*(kKMax+1)... ] normalised Legendre, m=0..kKMax, monomial coeffs
};
const Basis1D& basis(int k);

// Polynomial piece (monomial coefficients in the local variable y) of one
// hierarchical function; evaluation helpers return value / derivative in x.
struct HierFn {
    int level;   // 0-based hierarchical level (0 = Legendre level)
    int cell;    // 1-based
    int mode;    // 1-based
    double x0, xm, x1;          // support and midpoint (xm unused at level 0)
    double scale, dydx, shift;  // v(x) = scale * p(dydx*x - shift)
    double left[kKMax], right[kKMax];  // p on y<0 (or the whole piece at level 0) / y>0
    int k;
};
HierFn make_hier_fn(int k, int level, int cell, int mode);
// One-sided limits at x (side=+1 from the right, -1 from the left), periodic on [0,1).
double hier_value(const HierFn& f, double x, int side);
double hier_deriv(const HierFn& f, double x, int side);

// ----------------------------------------------------------- 1D operator ----
// Hierarchical periodic DG derivative with central flux, the operator that
// src/1d_derivative.jl:113-117 builds as hier2pos' * A * hier2pos.  Block
// sparse: one dense k x k block for every pair of (level, cell) blocks whose
// closed supports meet periodically.  Blocks are numbered in the reference's
// 1D vector order (levels 1..n+1, cells, modes).
struct DLF1D {
    int k = 0, n = 0;
    int nblocks = 0;                 // 2^n
    std::vector<int> blk_level;      // 1-based level of each block
    std::vector<int> blk_cell;       // 1-based cell
    std::vector<int32_t> rowptr;     // block-CSR by row block, nblocks+1
    std::vector<int32_t> colblk;     // column block per stored block (sorted per row)
    std::vector<double> val;         // k*k per stored block, [i][j] = D[rb*k+i][cb*k+j]
};
std::shared_ptr<const DLF1D> dlf1d(int k, int n);

// The 1D operator as the matrix-free kernels apply it: block CSR over the
// blocks that are not zero up to roundoff, each entry as an FP32 (hi, lo)
// pair, rows padded to rs floats.  A wavelet with k vanishing moments is
// orthogonal to the derivative of anything polynomial on its support, so a
// fine/coarse block pair vanishes unless the fine support touches a break of
// the coarse function; the reference's structural pattern keeps such blocks
// as numerical zeros (the plain CSR form keeps them too).  Blocks are dropped
// when their largest entry is below 1e-10 of the operator's largest entry;
// zero blocks sit below 1e-13 and kept ones above 1e-3 of it.  The kept
// blocks repeat (the periodic operator is translation invariant and the
// surviving fine/coarse pairs sit at a few positions relative to a break):
// k=3, n=7 keeps 1568 blocks but only 163 distinct ones, so the table stores
// distinct blocks once and each row lists (column block << 12 | block id).
struct MFOperator {
    int k = 0, n = 0, rs = 0, ndist = 0;
    std::vector<int32_t> rowptr;  // 2^n + 1
    std::vector<int32_t> ent;     // per row, sorted by column block
    std::vector<float> val;       // ndist blocks of k rows x rs floats
};
MFOperator mf_operator(int k, int n);                  // the 1D derivative, pruned
// The squared line operators B B (B = leading block of the pruned 1D
// operator for line length lm = 1..n+1), one block-CSR table per lm: row
// pointers of lm at rowptr[roff[lm - 1] ..], entries as in MFOperator, the
// distinct blocks shared by all lm.
struct MFSquareTables {
    int k = 0, n = 0, rs = 0, ndist = 0;
    std::vector<int32_t> roff;    // n + 1
    std::vector<int32_t> rowptr;  // sum over lm of 2^(lm-1) + 1
    std::vector<int32_t> ent;
    std::vector<float> val;
};
MFSquareTables mf_square_tables(int k, int n);
MFOperator mf_transform_table(int k, int n, int which);  // a nodal transform (see below)

// ------------------------------------------------------------ index map ----
// Sparse-grid coefficient layout of src/dg_vmethods.jl:102-142: level tuples
// in Julia CartesianIndices order (dimension 1 fastest), then cells, then modes.
struct SparseIndex {
    int D = 0, k = 0, n = 0, scheme = 0;
    int64_t N = 0, kD = 1;
    int nlev = 0;
    std::vector<int> levels;        // nlev x D, 1-based
    std::vector<int64_t> lev_off;   // nlev
    std::vector<int64_t> lev_cells; // nlev (product of cells)
    std::vector<int32_t> code2lev;  // (n+1)^D -> level block id or -1
    int64_t code(const int* L) const;
    int lookup_level(const int* L) const { return code2lev[code(L)]; }
    bool cut(const int* L) const;
};
SparseIndex make_index(int D, int k, int n, int scheme);
inline int64_t ncells(int L) { return int64_t(1) << (L > 2 ? L - 2 : 0); }
inline int log2cells(int L) { return L > 2 ? L - 2 : 0; }

// ------------------------------------------------------------------ CSR ----
struct CSR {
    int64_t m = 0, n = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    int64_t nnz() const { return rowptr.empty() ? 0 : rowptr.back(); }
};
CSR assemble_dd(const SparseIndex& ix, const DLF1D& op, int d);  // D_matrix(D, d + 1, k, n): d is 0-based
CSR spgemm_sum(const std::vector<const CSR*>& A);                  // sum_i A_i * A_i
CSR add_scaled(const std::vector<const CSR*>& A, const std::vector<double>& s);
CSR wave_rhs(const CSR& lap);                                                // wave_data
// periodic_pos_DLF_matrix(k, n) and its square (the position-basis operators
// of wave_evolve_1D); either pointer may be null
void pos_operators(int k, int n, CSR* dop, CSR* lap);

// ------------------------------------------------------ nodal transforms ----
// Maps between the modal (hierarchical), nodal and point bases of the Vlasov
// evolver (src/1d_nodal_basis.jl, src/multidim_nodal_basis.jl), k in {2,3,5}.
enum : int {
    TRANSFORM_MODAL_TO_NODAL = 0,
    TRANSFORM_NODAL_TO_POINTS = 1,
    TRANSFORM_POINTS_TO_NODAL = 2,
    TRANSFORM_NODAL_TO_MODAL = 3
};
CSR transform_1d(int k, int n, int which);                  // transform_1D
CSR transform_dd(const SparseIndex& ix, const CSR& T1);      // transform(D, k, n, mat_1D)
double nodal_point(int k, int L, int c, int m);                // collocation point of a point-basis index
std::vector<double> vlasov_velocity_points(const SparseIndex& ix, int Dx);  // 2 p_d - 1, Dx x N

// ------------------------------------------------------------ HDF5 out ----
// Root-group datasets (64-bit integers, doubles; scalars and 1D arrays) in an
// HDF5 file, as vlasov_evolve's vlasov.h5 holds them (h5write.cpp).
class H5Writer {
  public:
    explicit H5Writer(const std::string& path);
    ~H5Writer();
    H5Writer(const H5Writer&) = delete;
    H5Writer& operator=(const H5Writer&) = delete;
    void scalar_i64(const std::string& name, int64_t v);
    void array_i64(const std::string& name, const int64_t* v, int64_t n);
    void array_f64(const std::string& name, const double* v, int64_t n);
    void close();  // writes the metadata and the superblock

  private:
    static constexpr uint64_t kSuperblockBytes = 96;
    struct Entry {
        std::string name;
        bool is_float;
        int rank;
        int64_t n;
        uint64_t addr, bytes, oh;
    };
    void add(const std::string& name, bool is_float, int rank, int64_t n, const void* data);
    void put(const void* p, uint64_t n);  // p == nullptr: zeros
    void align8();
    std::string path_;
    std::FILE* f_ = nullptr;
    uint64_t pos_ = 0;
    std::vector<Entry> ents_;
};
void h5_write_csc(H5Writer& w, const std::string& name, const CSR& A);  // <name>.m, .n, .colptr, .rowval, .nzval

// ------------------------------------------------------ pencil schedule ----
// A pencil for dimension d fixes the levels of every other dimension; its
// elements are whole level blocks (L_-d, l) for l = 1..Lmax and form an
// m x R matrix: rows = 1D prefix of length k*2^(Lmax-1), columns = the other
// dimensions' cells and modes.
struct Pencil {
    int d;                 // 0-based dimension
    int lmax;              // 1-based max level along d
    int64_t R;             // columns
    int lp;                // log2 of prod_{q<d} cells_q
    std::vector<int64_t> blockoff;  // offset of level block (L_-d, l), l = 1..lmax
};
std::vector<Pencil> make_pencils(const SparseIndex& ix, int d);
// Appends, for every row (row block rb, mode i along d) of the pencil's 1D
// prefix, the pair (row offset, lc): element (row, column) of the pencil sits
// at row offset + a + (b << lc), with (a, b) the column's low and high parts
// (lc = log2 of the row level's cell count).
void pencil_rows(const Pencil& p, int k, int64_t kD, std::vector<int32_t>& out);

// The line operators of the pencils, for every line of lm = 1..levels levels
// (m = k 2^(lm-1) elements): the leading m x m block of the 1D operator, or
// its square (accumulated as spgemm_sum does, so the values are the same),
// as CSR over the line's 1D element index with sorted rows.  Table lm starts
// at rowptr[roff[lm-1]]; its row pointers index col/val directly.
struct LineTables {
    int k = 0, levels = 0;
    std::vector<int64_t> roff, rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
};
LineTables line_tables(const DLF1D& op, int levels, bool square);

void set_error(const std::string& msg);
}  // namespace sgdg
