// device_csr.h -- an assembled operator on the device: CSR arrays, the rows
// binned by length (lanes per row of the CSR kernels) and the long-row
// segments the kernels split rows of more than kCsrSplit entries into
// (kernels.cu).
#pragma once
#include <algorithm>
#include <memory>
#include <vector>

#include "device_util.h"
#include "engine.h"
#include "sgdg_core.h"

namespace sgdg {

struct DeviceCSR {
    DevBuf rowptr, col, val, bin_rows, long_row, long_seg, seg_begin, seg_end, partial;
    DevCSR d{};
};

constexpr int64_t kCsrSplit = 2048;  // entries a row group sums directly

// bin of a row of L <= kCsrSplit entries: the fewest lanes 2^b (up to 32)
// that give each lane at most `per_lane` entries (fewer lanes per row: fewer
// FP64 additions in the lane reduction, which on GB300 cost as much as the
// FMAs).  32 entries per lane suit single-vector passes: the 256-solve wave
// batch steps in 20.1 ms against 26.2 at 16 and 31.8 at 8 (its rows hold ~96
// entries); the nodal transforms, passed over four vectors at once, keep 8
// (the Vlasov plain step 2.60 ms against 2.66 at 16 and 2.67 at 32).
constexpr int kCsrLaneEntries = 32;
constexpr int kCsrLaneEntriesMulti = 8;
inline int csr_bin(int64_t L, int per_lane) {
    int b = 0;
    while (b + 1 < kCsrBins && (int64_t(per_lane) << b) < L) b++;
    return b;
}

// Fills D.d from D's buffers (already holding rowptr, col, val for m rows)
// and builds the long-row segments from the host copy of the row pointers.
inline void finish_device_csr(DeviceCSR& D, const std::vector<int64_t>& rowptr, int64_t m, cudaStream_t st,
                              int per_lane = kCsrLaneEntries) {
    const int64_t nnz = rowptr[m];
    D.d.m = m;
    D.d.nnz = nnz;
    D.d.rowptr = D.rowptr.as<int64_t>();
    D.d.col = D.col.as<int32_t>();
    D.d.val = D.val.as<double>();
    // rows by bin (counting sort, ascending rows within a bin) and the
    // blocks of 256 threads each bin takes
    std::vector<int64_t> cnt(kCsrBins + 1, 0);
    for (int64_t r = 0; r < m; r++) {
        const int64_t L = rowptr[r + 1] - rowptr[r];
        if (L <= kCsrSplit) cnt[csr_bin(L, per_lane) + 1]++;
    }
    int64_t blocks = 0;
    for (int b = 0; b < kCsrBins; b++) {
        D.d.bin_block[b] = (int)blocks;
        blocks += (cnt[b + 1] * (int64_t(1) << b) + 255) / 256;
        cnt[b + 1] += cnt[b];
        D.d.bin_first[b] = cnt[b];
    }
    if (blocks > (int64_t(1) << 30)) throw Error(SGDG_EINVAL, "operator too large for the CSR kernels");
    D.d.bin_block[kCsrBins] = (int)blocks;
    D.d.bin_first[kCsrBins] = cnt[kCsrBins];
    std::vector<int32_t> rows((size_t)cnt[kCsrBins]);
    {
        std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
        for (int64_t r = 0; r < m; r++) {
            const int64_t L = rowptr[r + 1] - rowptr[r];
            if (L <= kCsrSplit) rows[(size_t)fill[csr_bin(L, per_lane)]++] = (int32_t)r;
        }
    }
    D.d.bin_rows = nullptr;
    if (!rows.empty()) {
        D.bin_rows = upload(rows, st);
        D.d.bin_rows = D.bin_rows.as<int32_t>();
    }
    std::vector<int32_t> lrow, lseg(1, 0);
    std::vector<int64_t> sb, se;
    for (int64_t r = 0; r < m; r++) {
        const int64_t b = rowptr[r], e = rowptr[r + 1];
        if (e - b <= kCsrSplit) continue;
        lrow.push_back((int32_t)r);
        for (int64_t p = b; p < e; p += kCsrSplit) {
            sb.push_back(p);
            se.push_back(std::min(e, p + kCsrSplit));
        }
        lseg.push_back((int32_t)sb.size());
    }
    D.d.split = kCsrSplit;
    D.d.nlong = (int64_t)lrow.size();
    D.d.nseg = (int64_t)sb.size();
    if (!lrow.empty()) {
        D.long_row = upload(lrow, st);
        D.long_seg = upload(lseg, st);
        D.seg_begin = upload(sb, st);
        D.seg_end = upload(se, st);
        D.partial.alloc(sizeof(double) * sb.size() * kCsrMaxVec);
        D.d.long_row = D.long_row.as<int32_t>();
        D.d.long_seg = D.long_seg.as<int32_t>();
        D.d.seg_begin = D.seg_begin.as<int64_t>();
        D.d.seg_end = D.seg_end.as<int64_t>();
        D.d.partial = D.partial.as<double>();
    }
}

inline std::unique_ptr<DeviceCSR> to_device(const CSR& A, cudaStream_t st) {
    auto D = std::make_unique<DeviceCSR>();
    D->rowptr = upload(A.rowptr, st);
    D->col = upload(A.col, st);
    D->val = upload(A.val, st);
    finish_device_csr(*D, A.rowptr, A.m, st);
    return D;
}

// The plain-form operators assembled on the GPU (gpu_assemble.cu): which =
// 1..D for D_d, SGDG_OP_LAPLACIAN, SGDG_OP_WAVE_RHS; the same stored entries
// and values as the host assembly (assemble.cpp).
std::unique_ptr<DeviceCSR> gpu_operator(const SparseIndex& ix, const DLF1D& dlf, int which, cudaStream_t st,
                                        int per_lane = kCsrLaneEntries);
// sum_d s[d] D_d over the union of patterns (the plain advection operator)
std::unique_ptr<DeviceCSR> gpu_scaled_sum(const SparseIndex& ix, const DLF1D& dlf, const double* s, cudaStream_t st);
// The D-dim restricted Kronecker product of the 1D transform T1 (the same
// entries, order and values as transform_dd, nodal.cpp)
std::unique_ptr<DeviceCSR> gpu_transform(const SparseIndex& ix, const CSR& T1, cudaStream_t st);
// host copy of a device operator
CSR download_csr(const DeviceCSR& A, cudaStream_t st);

}  // namespace sgdg
