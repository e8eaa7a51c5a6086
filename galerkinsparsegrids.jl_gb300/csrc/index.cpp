// index.cpp -- sparse-grid coefficient layout and pencil schedules.
//
// Layout (kept identical to the reference so coefficient vectors cross the
// boundary without permutation): level tuples in Julia CartesianIndices order
// with dimension 1 fastest, skipping tuples with sum(L) > n + D for the
// sparse scheme (src/schemes.jl:21-27); inside a level block, cells then
// modes, each column-major (src/dg_vmethods.jl:102-142).
#include "sgdg_core.h"

namespace sgdg {

int64_t SparseIndex::code(const int* L) const {
    int64_t c = 0;
    for (int q = D - 1; q >= 0; q--) c = c * (n + 1) + (L[q] - 1);
    return c;
}

bool SparseIndex::cut(const int* L) const {
    if (scheme == 1) return false;
    int s = 0;
    for (int q = 0; q < D; q++) s += L[q];
    return s > n + D;
}

SparseIndex make_index(int D, int k, int n, int scheme) {
    if (D < 1 || D > kDMax) throw Error(1, "D must be in 1..8");
    if (k < 1 || k > kKMax) throw Error(1, "k must be in 1..10 (K_max)");
    if (n < 0 || n > 20) throw Error(1, "n out of range");
    if (scheme != 0 && scheme != 1) throw Error(1, "scheme must be sparse (0) or full (1)");
    SparseIndex ix;
    ix.D = D;
    ix.k = k;
    ix.n = n;
    ix.scheme = scheme;
    ix.kD = 1;
    for (int q = 0; q < D; q++) ix.kD *= k;
    int64_t ncodes = 1;
    for (int q = 0; q < D; q++) {
        ncodes *= (n + 1);
        if (ncodes > (int64_t(1) << 26)) throw Error(1, "(n+1)^D too large");
    }
    ix.code2lev.assign(ncodes, -1);
    int L[kDMax];
    int64_t off = 0;
    for (int64_t c = 0; c < ncodes; c++) {
        int64_t t = c;
        for (int q = 0; q < D; q++) {
            L[q] = int(t % (n + 1)) + 1;
            t /= (n + 1);
        }
        if (ix.cut(L)) continue;
        int64_t cells = 1;
        for (int q = 0; q < D; q++) cells *= ncells(L[q]);
        ix.code2lev[c] = ix.nlev;
        for (int q = 0; q < D; q++) ix.levels.push_back(L[q]);
        ix.lev_off.push_back(off);
        ix.lev_cells.push_back(cells);
        ix.nlev++;
        off += cells * ix.kD;
        if (off > (int64_t(1) << 31) - 1) throw Error(2, "state larger than 2^31 coefficients");
    }
    ix.N = off;
    return ix;
}

std::vector<Pencil> make_pencils(const SparseIndex& ix, int d) {
    std::vector<Pencil> out;
    const int D = ix.D;
    int L[kDMax];
    // enumerate level blocks whose level along d is 1: each starts one pencil
    for (int b = 0; b < ix.nlev; b++) {
        const int* Lb = &ix.levels[(size_t)b * D];
        if (Lb[d] != 1) continue;
        Pencil p;
        p.d = d;
        for (int q = 0; q < D; q++) L[q] = Lb[q];
        int lmax = 0;
        for (int l = 1; l <= ix.n + 1; l++) {
            L[d] = l;
            if (ix.cut(L)) break;
            p.blockoff.push_back(ix.lev_off[ix.lookup_level(L)]);
            lmax = l;
        }
        p.lmax = lmax;
        int64_t R = 1;
        int lp = 0;
        for (int q = 0; q < D; q++) {
            if (q == d) continue;
            R *= ncells(Lb[q]) * ix.k;
            if (q < d) lp += log2cells(Lb[q]);
        }
        p.R = R;
        p.lp = lp;
        out.push_back(std::move(p));
    }
    return out;
}

void pencil_rows(const Pencil& p, int k, int64_t kD, std::vector<int32_t>& out) {
    int64_t kd1 = 1;
    for (int q = 0; q < p.d; q++) kd1 *= k;
    const int nrb = 1 << (p.lmax - 1);
    for (int rb = 0; rb < nrb; rb++) {
        // row block rb of the pencil's 1D prefix: level l, cell cd0 within the level
        int l = 1;
        while (l < 32 && (rb >> (l - 1)) != 0) l++;
        const int64_t cd0 = l >= 2 ? rb - (1 << (l - 2)) : 0;
        const int lc = l > 2 ? l - 2 : 0;
        for (int i = 0; i < k; i++) {
            out.push_back((int32_t)(p.blockoff[l - 1] + kD * (cd0 << p.lp) + i * kd1));
            out.push_back(lc);
        }
    }
}

}  // namespace sgdg
