// h5write.cpp -- the output file of vlasov_evolve (src/pdes.jl:145-163 writes
// the operators, :217-223 the solution): root-group datasets of 64-bit signed
// integers and IEEE doubles, scalars and 1D arrays, under the reference's
// names.  The reference writes through JLD2, whose files are HDF5 files; this
// writer produces an HDF5 file directly, from the published HDF5 File Format
// Specification, with the simplest structures it allows:
//   * a version 0 superblock at offset 0 (8-byte offsets and lengths);
//   * an old-style root group: a version 1 object header holding a symbol
//     table message, a version 1 group B-tree with a single leaf, one symbol
//     table node with every entry (group leaf node K is raised to hold them
//     all) and a local heap with the names;
//   * per dataset a version 1 object header with a version 1 dataspace, a
//     version 1 fixed-point or floating-point datatype, a version 2 fill value
//     (none defined) and a version 3 contiguous layout message.
// Array data is written first, as it is added; the metadata and the
// superblock when the file is closed.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgdg.h"
#include "sgdg_core.h"

namespace sgdg {
namespace {

constexpr uint64_t kUndef = ~uint64_t(0);
constexpr int kInternalK = 16;  // group internal node K (the library default)

struct Bytes {
    std::vector<uint8_t> b;
    void u8(unsigned v) { b.push_back(uint8_t(v)); }
    void le(uint64_t v, int n) {
        for (int i = 0; i < n; i++) b.push_back(uint8_t(v >> (8 * i)));
    }
    void raw(const void* p, size_t n) {
        const uint8_t* q = static_cast<const uint8_t*>(p);
        b.insert(b.end(), q, q + n);
    }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8() { zeros((8 - b.size() % 8) % 8); }
};

// one object header message: type, data padded to a multiple of 8 bytes
void message(Bytes& oh, unsigned type, unsigned flags, const Bytes& data) {
    Bytes d = data;
    d.pad8();
    oh.le(type, 2);
    oh.le(d.b.size(), 2);
    oh.u8(flags);
    oh.zeros(3);
    oh.raw(d.b.data(), d.b.size());
}

// version 1 object header around `msgs` (count messages)
Bytes object_header(const Bytes& msgs, int count) {
    Bytes oh;
    oh.u8(1);  // version
    oh.u8(0);
    oh.le(count, 2);
    oh.le(1, 4);  // reference count
    oh.le(msgs.b.size(), 4);
    oh.zeros(4);  // messages start 8-byte aligned
    oh.raw(msgs.b.data(), msgs.b.size());
    return oh;
}

}  // namespace

H5Writer::H5Writer(const std::string& path) : path_(path) {
    f_ = std::fopen(path.c_str(), "wb");
    if (!f_) throw Error(SGDG_EIO, "cannot open " + path + " for writing");
    pos_ = 0;
    put(nullptr, kSuperblockBytes);  // the superblock goes here on close
}

H5Writer::~H5Writer() {
    if (f_) std::fclose(f_);
}

void H5Writer::put(const void* p, uint64_t n) {
    static const uint8_t z[4096] = {};
    uint64_t left = n;
    const uint8_t* q = static_cast<const uint8_t*>(p);
    while (left > 0) {
        const size_t c = (size_t)std::min<uint64_t>(left, p ? left : sizeof(z));
        if (std::fwrite(p ? q : z, 1, c, f_) != c) throw Error(SGDG_EIO, "write failed: " + path_);
        if (p) q += c;
        left -= c;
    }
    pos_ += n;
}

void H5Writer::align8() {
    if (pos_ % 8) put(nullptr, 8 - pos_ % 8);
}

void H5Writer::add(const std::string& name, bool is_float, int rank, int64_t n, const void* data) {
    if (name.empty() || name.find('/') != std::string::npos || name.find('\0') != std::string::npos)
        throw Error(SGDG_EINVAL, "bad dataset name");
    for (const Entry& e : ents_)
        if (e.name == name) throw Error(SGDG_EINVAL, "duplicate dataset " + name);
    if (n < 0) throw Error(SGDG_EINVAL, "negative length");
    Entry e{name, is_float, rank, n, kUndef, 8 * (uint64_t)n, 0};
    if (e.bytes > 0) {
        align8();
        e.addr = pos_;
        put(data, e.bytes);
    }
    ents_.push_back(e);
}

void H5Writer::scalar_i64(const std::string& name, int64_t v) { add(name, false, 0, 1, &v); }
void H5Writer::array_i64(const std::string& name, const int64_t* v, int64_t n) { add(name, false, 1, n, v); }
void H5Writer::array_f64(const std::string& name, const double* v, int64_t n) { add(name, true, 1, n, v); }

void H5Writer::close() {
    if (!f_) return;
    const size_t ne = ents_.size();
    // group leaf node K: one symbol table node of 2K entries holds every name
    const uint64_t leafk = std::max<uint64_t>(4, (ne + 1) / 2);
    if (leafk > 65535) throw Error(SGDG_EUNSUPPORTED, "more than 131,070 datasets in one file");

    // dataset object headers
    for (Entry& e : ents_) {
        Bytes msgs, m;
        // dataspace, version 1: rank 0 is a scalar
        m.u8(1);
        m.u8(e.rank);
        m.u8(0);
        m.u8(0);
        m.zeros(4);
        if (e.rank == 1) m.le(e.n, 8);
        message(msgs, 0x0001, 0, m);
        m.b.clear();
        // datatype, version 1: 64-bit signed little-endian integer or IEEE double
        if (e.is_float) {
            m.u8(0x11);  // version 1, class 1 (floating point)
            m.u8(0x20);  // little endian, no padding, mantissa normalisation "implied"
            m.u8(63);    // sign bit
            m.u8(0);
            m.le(8, 4);
            m.le(0, 2);   // bit offset
            m.le(64, 2);  // precision
            m.u8(52);     // exponent location
            m.u8(11);     // exponent size
            m.u8(0);      // mantissa location
            m.u8(52);     // mantissa size
            m.le(1023, 4);
        } else {
            m.u8(0x10);  // version 1, class 0 (fixed point)
            m.u8(0x08);  // little endian, no padding, signed
            m.u8(0);
            m.u8(0);
            m.le(8, 4);
            m.le(0, 2);
            m.le(64, 2);
        }
        message(msgs, 0x0003, 1, m);
        m.b.clear();
        // fill value, version 2: space allocated early, fill written only if
        // one is set (write time 2), none set
        m.u8(2);
        m.u8(1);
        m.u8(2);
        m.u8(0);
        message(msgs, 0x0005, 1, m);
        m.b.clear();
        // layout, version 3: contiguous
        m.u8(3);
        m.u8(1);
        m.le(e.addr, 8);
        m.le(e.bytes, 8);
        message(msgs, 0x0008, 0, m);
        const Bytes oh = object_header(msgs, 4);
        align8();
        e.oh = pos_;
        put(oh.b.data(), oh.b.size());
    }

    // names sorted as the B-tree compares them (byte-wise)
    std::vector<size_t> order(ne);
    for (size_t i = 0; i < ne; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return std::strcmp(ents_[a].name.c_str(), ents_[b].name.c_str()) < 0;
    });

    // local heap: "" at offset 0, the names (null-terminated, 8-byte aligned),
    // then one free block (next = 1: the last block; its size)
    Bytes heap;
    heap.zeros(8);
    std::vector<uint64_t> name_off(ne);
    for (size_t i : order) {
        name_off[i] = heap.b.size();
        heap.raw(ents_[i].name.c_str(), ents_[i].name.size() + 1);
        heap.pad8();
    }
    const uint64_t free_off = heap.b.size();
    heap.le(1, 8);
    heap.le(16, 8);
    align8();
    const uint64_t heap_addr = pos_;
    {
        Bytes h;
        h.raw("HEAP", 4);
        h.u8(0);
        h.zeros(3);
        h.le(heap.b.size(), 8);
        h.le(free_off, 8);
        h.le(heap_addr + 32, 8);
        put(h.b.data(), h.b.size());
        put(heap.b.data(), heap.b.size());
    }

    // symbol table node with every entry, sized for 2K entries
    align8();
    const uint64_t snod_addr = pos_;
    {
        Bytes s;
        s.raw("SNOD", 4);
        s.u8(1);
        s.u8(0);
        s.le(ne, 2);
        for (size_t i : order) {
            s.le(name_off[i], 8);
            s.le(ents_[i].oh, 8);
            s.le(0, 4);  // cache type: nothing cached
            s.zeros(4 + 16);
        }
        s.zeros((2 * leafk - ne) * 40);
        put(s.b.data(), s.b.size());
    }

    // group B-tree: one leaf node pointing at the symbol table node, sized for
    // 2K children; keys are heap offsets ("" then the last name of the child)
    align8();
    const uint64_t btree_addr = pos_;
    {
        Bytes t;
        t.raw("TREE", 4);
        t.u8(0);  // group node
        t.u8(0);  // leaf level
        t.le(1, 2);
        t.le(kUndef, 8);
        t.le(kUndef, 8);
        t.le(0, 8);
        t.le(snod_addr, 8);
        t.le(ne ? name_off[order.back()] : 0, 8);
        t.zeros((2 * kInternalK - 1) * 16);
        put(t.b.data(), t.b.size());
    }

    // root group object header: the symbol table message
    align8();
    const uint64_t root_oh = pos_;
    {
        Bytes msgs, m;
        m.le(btree_addr, 8);
        m.le(heap_addr, 8);
        message(msgs, 0x0011, 0, m);
        const Bytes oh = object_header(msgs, 1);
        put(oh.b.data(), oh.b.size());
    }
    const uint64_t eof = pos_;

    // superblock, version 0
    Bytes sb;
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    sb.raw(sig, 8);
    sb.u8(0);  // superblock version
    sb.u8(0);  // free-space storage version
    sb.u8(0);  // root group symbol table entry version
    sb.u8(0);
    sb.u8(0);  // shared header message format version
    sb.u8(8);  // size of offsets
    sb.u8(8);  // size of lengths
    sb.u8(0);
    sb.le(leafk, 2);
    sb.le(kInternalK, 2);
    sb.le(0, 4);  // consistency flags
    sb.le(0, 8);  // base address
    sb.le(kUndef, 8);
    sb.le(eof, 8);
    sb.le(kUndef, 8);
    sb.le(0, 8);  // root entry: name offset
    sb.le(root_oh, 8);
    sb.le(1, 4);  // cache type 1: B-tree and heap addresses in the scratch pad
    sb.le(0, 4);
    sb.le(btree_addr, 8);
    sb.le(heap_addr, 8);
    if (sb.b.size() != kSuperblockBytes) throw Error(SGDG_EINVAL, "internal: superblock size");
    if (std::fseek(f_, 0, SEEK_SET) != 0 || std::fwrite(sb.b.data(), 1, sb.b.size(), f_) != sb.b.size())
        throw Error(SGDG_EIO, "write failed: " + path_);
    const int rc = std::fclose(f_);
    f_ = nullptr;
    if (rc != 0) throw Error(SGDG_EIO, "close failed: " + path_);
}

// CSC fields of A (src/pdes.jl:149-155): m, n, colptr and rowval 1-based
void h5_write_csc(H5Writer& w, const std::string& name, const CSR& A) {
    const int64_t m = A.m, n = A.n, nnz = A.nnz();
    std::vector<int64_t> colptr((size_t)n + 1, 0), rowval((size_t)nnz);
    std::vector<double> nzval((size_t)nnz);
    for (int64_t q = 0; q < nnz; q++) colptr[(size_t)A.col[(size_t)q] + 1]++;
    for (int64_t j = 0; j < n; j++) colptr[(size_t)j + 1] += colptr[(size_t)j];
    std::vector<int64_t> next(colptr.begin(), colptr.end() - 1);
    for (int64_t r = 0; r < m; r++)  // rows ascending: each column's rows come out sorted
        for (int64_t q = A.rowptr[(size_t)r]; q < A.rowptr[(size_t)r + 1]; q++) {
            const int64_t at = next[(size_t)A.col[(size_t)q]]++;
            rowval[(size_t)at] = r + 1;
            nzval[(size_t)at] = A.val[(size_t)q];
        }
    for (int64_t& c : colptr) c += 1;
    w.scalar_i64(name + ".m", m);
    w.scalar_i64(name + ".n", n);
    w.array_i64(name + ".colptr", colptr.data(), n + 1);
    w.array_i64(name + ".rowval", rowval.data(), nnz);
    w.array_f64(name + ".nzval", nzval.data(), nnz);
}

}  // namespace sgdg
