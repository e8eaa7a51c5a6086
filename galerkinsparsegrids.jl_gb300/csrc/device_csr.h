// device_csr.h -- an assembled operator on the device: CSR arrays plus the
// long-row segments the SpMV kernels split rows of more than kCsrSplit
// entries into (kernels.cu).
#pragma once
#include <algorithm>
#include <memory>
#include <vector>

#include "device_util.h"
#include "engine.h"
#include "sgdg_core.h"

namespace sgdg {

struct DeviceCSR {
    DevBuf rowptr, col, val, long_row, long_seg, seg_begin, seg_end, partial;
    DevCSR d{};
};

constexpr int64_t kCsrSplit = 2048;  // entries a row group sums directly

// lanes per row of the CSR kernels, from the mean row length
inline int pick_vs(int64_t m, int64_t nnz) {
    const double avg = m ? double(nnz) / double(m) : 0.0;
    if (avg <= 2) return 1;
    if (avg <= 4) return 2;
    if (avg <= 10) return 4;
    if (avg <= 24) return 8;
    if (avg <= 48) return 16;
    return 32;
}

// Fills D.d from D's buffers (already holding rowptr, col, val for m rows)
// and builds the long-row segments from the host copy of the row pointers.
inline void finish_device_csr(DeviceCSR& D, const std::vector<int64_t>& rowptr, int64_t m, cudaStream_t st) {
    const int64_t nnz = rowptr[m];
    D.d.m = m;
    D.d.nnz = nnz;
    D.d.rowptr = D.rowptr.as<int64_t>();
    D.d.col = D.col.as<int32_t>();
    D.d.val = D.val.as<double>();
    D.d.vs = pick_vs(m, nnz);
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
        D.partial.alloc(sizeof(double) * sb.size());
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
std::unique_ptr<DeviceCSR> gpu_operator(const SparseIndex& ix, const DLF1D& dlf, int which, cudaStream_t st);
// sum_d s[d] D_d over the union of patterns (the plain advection operator)
std::unique_ptr<DeviceCSR> gpu_scaled_sum(const SparseIndex& ix, const DLF1D& dlf, const double* s, cudaStream_t st);
// The D-dim restricted Kronecker product of the 1D transform T1 (the same
// entries, order and values as transform_dd, nodal.cpp)
std::unique_ptr<DeviceCSR> gpu_transform(const SparseIndex& ix, const CSR& T1, cudaStream_t st);
// host copy of a device operator
CSR download_csr(const DeviceCSR& A, cudaStream_t st);

}  // namespace sgdg
