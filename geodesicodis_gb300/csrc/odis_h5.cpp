// The run's DATA/data.h5 container (src/outFiles.cpp:138-823) written without
// the HDF5 library, which this library does not depend on.
//
// The file has the structure that the HDF5 library writes with default property
// lists (H5Fcreate / H5Dcreate with H5P_DEFAULT, as the reference calls them),
// restated from the published HDF5 file-format specification:
//   * superblock version 0, 8-byte offsets and lengths, group leaf node K 4,
//     group internal node K 16;
//   * the root group as a symbol table: a version-1 object header holding a
//     symbol-table message, a version-1 B-tree of type 0 (one leaf node), symbol
//     nodes of at most 2 x 4 entries in name order, and a local heap with the
//     link names and one trailing free block (whose next-block offset is 1, the
//     library's end of list);
//   * per dataset a version-1 object header with dataspace (version 1, current
//     and maximum extents equal), IEEE float32 little-endian datatype, fill value
//     (version 2, default fill), contiguous layout (version 3) and modification
//     time messages, padded with a null message to 256 bytes;
//   * the datasets' contiguous storage, allocated when the file is created and
//     zero-filled, so rows not yet written read as the default fill value 0.
// Rows are then written in place as the run produces them, like the reference's
// per-dump hyperslab writes.
#include "../../include/odis_gpu.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <unistd.h>
#include <vector>

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;                  // group leaf node K: a symbol node holds <= 2K entries
constexpr int kInternalK = 16;             // group internal node K: a B-tree node has <= 2K children
constexpr int kSuperblock = 96;
constexpr int kRootHeader = 16 + 8 + 16;   // prefix + symbol-table message
constexpr int kBtreeNode = 24 + 2 * kInternalK * 8 + (2 * kInternalK + 1) * 8;
constexpr int kHeapHeader = 32;
constexpr int kSymbolNode = 8 + 2 * kLeafK * 40;
constexpr int kDatasetHeaderBody = 256;
constexpr int kDatasetHeader = 16 + kDatasetHeaderBody;

struct Dataset {
    std::string name;
    int rank = 0;
    uint64_t dims[2] = {0, 0};
    uint64_t heap_off = 0, header = 0, data = 0, bytes = 0, row_bytes = 0, rows = 0;
};

struct Bytes {
    std::vector<uint8_t> b;
    void u8(unsigned v) { b.push_back((uint8_t)v); }
    void u16(unsigned v) { for (int i = 0; i < 2; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void u32(uint32_t v) { for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void tag(const char* s) { for (int i = 0; i < 4; i++) b.push_back((uint8_t)s[i]); }
    void pad_to(size_t n) { if (b.size() < n) zeros(n - b.size()); }
};

// version-1 object header message: type, body size (a multiple of 8), flags, reserved
void message(Bytes& o, unsigned type, const Bytes& body, unsigned flags)
{
    const size_t n = (body.b.size() + 7) / 8 * 8;
    o.u16(type);
    o.u16((unsigned)n);
    o.u8(flags);
    o.zeros(3);
    o.b.insert(o.b.end(), body.b.begin(), body.b.end());
    o.zeros(n - body.b.size());
}

// symbol table entry: link name offset, object header address, cache type, reserved, scratch pad
void symbol_entry(Bytes& o, uint64_t name_off, uint64_t header, unsigned cache, uint64_t btree, uint64_t heap)
{
    o.u64(name_off);
    o.u64(header);
    o.u32(cache);
    o.u32(0);
    if (cache == 1) { o.u64(btree); o.u64(heap); }
    else o.zeros(16);
}

void dataset_header(Bytes& o, const Dataset& d, uint32_t mtime)
{
    const size_t start = o.b.size();
    o.u8(1); o.u8(0); o.u16(6); o.u32(1); o.u32(kDatasetHeaderBody); o.zeros(4);
    Bytes sp;                                         // dataspace, version 1, maximum extents present
    sp.u8(1); sp.u8((unsigned)d.rank); sp.u8(1); sp.u8(0); sp.u32(0);
    for (int r = 0; r < d.rank; r++) sp.u64(d.dims[r]);
    for (int r = 0; r < d.rank; r++) sp.u64(d.dims[r]);
    message(o, 0x0001, sp, 0);
    Bytes ty;                                         // IEEE float32, little-endian, implied mantissa MSB
    ty.u8(0x11); ty.u8(0x20); ty.u8(31); ty.u8(0); ty.u32(4);
    ty.u16(0); ty.u16(32); ty.u8(23); ty.u8(8); ty.u8(0); ty.u8(23); ty.u32(127);
    message(o, 0x0003, ty, 1);
    Bytes fv;                                         // fill value, version 2: late allocation, write if set, default
    fv.u8(2); fv.u8(2); fv.u8(2); fv.u8(1); fv.u32(0);
    message(o, 0x0005, fv, 1);
    Bytes ly;                                         // layout, version 3, contiguous
    ly.u8(3); ly.u8(1); ly.u64(d.data); ly.u64(d.bytes);
    message(o, 0x0008, ly, 0);
    Bytes mt;                                         // modification time, version 1
    mt.u8(1); mt.zeros(3); mt.u32(mtime);
    message(o, 0x0012, mt, 0);
    const size_t used = o.b.size() - start - 16;
    Bytes nil;                                        // null message over the rest of the header
    nil.zeros(kDatasetHeaderBody - used - 8);
    message(o, 0x0000, nil, 0);
}

}  // namespace

struct odis_h5 {
    FILE* f = nullptr;
    std::vector<Dataset> ds;
};

extern "C" odis_status odis_h5_create(const char* path, int n, const char* const* names, const int* ranks,
                                      const long long* dims, odis_h5** out)
{
    if (!out) return ODIS_ERR_ARG;
    *out = nullptr;
    if (!path || !names || !ranks || !dims || n < 1 || n > 2 * kLeafK * 2 * kInternalK) return ODIS_ERR_ARG;
    std::vector<Dataset> ds(n);
    for (int k = 0; k < n; k++) {
        if (!names[k] || !names[k][0] || (ranks[k] != 1 && ranks[k] != 2)) return ODIS_ERR_ARG;
        ds[k].name = names[k];
        ds[k].rank = ranks[k];
        for (int r = 0; r < ranks[k]; r++) {
            if (dims[2 * k + r] < 1) return ODIS_ERR_ARG;
            ds[k].dims[r] = (uint64_t)dims[2 * k + r];
        }
        ds[k].rows = ds[k].dims[0];
        ds[k].row_bytes = 4 * (ds[k].rank == 2 ? ds[k].dims[1] : 1);
        ds[k].bytes = ds[k].rows * ds[k].row_bytes;
    }
    // link names in byte order (the order of the symbol nodes and of the B-tree keys)
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return std::strcmp(ds[a].name.c_str(), ds[b].name.c_str()) < 0; });
    for (int k = 1; k < n; k++)
        if (ds[order[k]].name == ds[order[k - 1]].name) return ODIS_ERR_ARG;
    // local heap data: offset 0 is the empty name, then each name NUL-terminated, 8-byte aligned
    Bytes heap;
    heap.zeros(8);
    for (int k : order) {
        ds[k].heap_off = heap.b.size();
        heap.b.insert(heap.b.end(), ds[k].name.begin(), ds[k].name.end());
        heap.u8(0);
        heap.pad_to((heap.b.size() + 7) / 8 * 8);
    }
    // a trailing free block, as the library leaves one: offset of the next free
    // block (1 = none) and this block's size
    const uint64_t free_off = heap.b.size();
    heap.u64(1);
    heap.u64(16);
    const int nsnod = (n + 2 * kLeafK - 1) / (2 * kLeafK);
    const uint64_t a_root = kSuperblock, a_btree = a_root + kRootHeader, a_heap = a_btree + kBtreeNode;
    const uint64_t a_heap_data = a_heap + kHeapHeader, a_snod = a_heap_data + heap.b.size();
    const uint64_t a_headers = a_snod + (uint64_t)nsnod * kSymbolNode;
    uint64_t a = a_headers + (uint64_t)n * kDatasetHeader;
    for (int k = 0; k < n; k++) ds[k].header = a_headers + (uint64_t)k * kDatasetHeader;
    for (int k = 0; k < n; k++) {
        a = (a + 7) / 8 * 8;
        ds[k].data = a;
        a += ds[k].bytes;
    }
    const uint64_t eof = a;

    Bytes o;
    // superblock, version 0
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    o.b.insert(o.b.end(), sig, sig + 8);
    o.u8(0); o.u8(0); o.u8(0); o.u8(0); o.u8(0); o.u8(8); o.u8(8); o.u8(0);
    o.u16(kLeafK); o.u16(kInternalK); o.u32(0);
    o.u64(0); o.u64(kUndef); o.u64(eof); o.u64(kUndef);
    symbol_entry(o, 0, a_root, 1, a_btree, a_heap);
    // root group object header: one symbol-table message
    o.u8(1); o.u8(0); o.u16(1); o.u32(1); o.u32(24); o.zeros(4);
    Bytes st;
    st.u64(a_btree); st.u64(a_heap);
    message(o, 0x0011, st, 0);
    // B-tree leaf node over the symbol nodes; key i+1 = the last name of symbol node i
    o.tag("TREE"); o.u8(0); o.u8(0); o.u16((unsigned)nsnod); o.u64(kUndef); o.u64(kUndef);
    o.u64(0);
    for (int s = 0; s < nsnod; s++) {
        const int last = std::min(n, (s + 1) * 2 * kLeafK) - 1;
        o.u64(a_snod + (uint64_t)s * kSymbolNode);
        o.u64(ds[order[last]].heap_off);
    }
    o.pad_to(a_heap);
    // local heap, version 0: data segment size, head of the free list, data segment address
    o.tag("HEAP"); o.u8(0); o.zeros(3); o.u64(heap.b.size()); o.u64(free_off); o.u64(a_heap_data);
    o.b.insert(o.b.end(), heap.b.begin(), heap.b.end());
    // symbol nodes, version 1
    for (int s = 0; s < nsnod; s++) {
        const int lo = s * 2 * kLeafK, hi = std::min(n, lo + 2 * kLeafK);
        const size_t start = o.b.size();
        o.tag("SNOD"); o.u8(1); o.u8(0); o.u16((unsigned)(hi - lo));
        for (int j = lo; j < hi; j++) symbol_entry(o, ds[order[j]].heap_off, ds[order[j]].header, 0, 0, 0);
        o.pad_to(start + kSymbolNode);
    }
    const uint32_t mtime = (uint32_t)std::time(nullptr);
    for (int k = 0; k < n; k++) dataset_header(o, ds[k], mtime);
    if (o.b.size() != a_headers + (uint64_t)n * kDatasetHeader) return ODIS_ERR_ARG;

    FILE* f = std::fopen(path, "wb+");
    if (!f) return ODIS_ERR_IO;
    bool ok = std::fwrite(o.b.data(), 1, o.b.size(), f) == o.b.size();
    ok = ok && std::fflush(f) == 0 && ftruncate(fileno(f), (off_t)eof) == 0;   // zero-filled storage
    if (!ok) {
        std::fclose(f);
        return ODIS_ERR_IO;
    }
    odis_h5* h = new odis_h5;
    h->f = f;
    h->ds = std::move(ds);
    *out = h;
    return ODIS_OK;
}

extern "C" odis_status odis_h5_write_rows(odis_h5* h, int k, long long row0, long long nrows, const float* data)
{
    if (!h || !h->f || k < 0 || k >= (int)h->ds.size() || row0 < 0 || nrows < 0 || (nrows && !data))
        return ODIS_ERR_ARG;
    const Dataset& d = h->ds[k];
    if ((uint64_t)(row0 + nrows) > d.rows) return ODIS_ERR_ARG;
    if (nrows == 0) return ODIS_OK;
    const size_t bytes = (size_t)(nrows * d.row_bytes);
    if (fseeko(h->f, (off_t)(d.data + (uint64_t)row0 * d.row_bytes), SEEK_SET) != 0) return ODIS_ERR_IO;
    // the file stores little-endian float32; the host is little-endian (x86-64, aarch64)
    return std::fwrite(data, 1, bytes, h->f) == bytes ? ODIS_OK : ODIS_ERR_IO;
}

extern "C" odis_status odis_h5_close(odis_h5* h)
{
    if (!h) return ODIS_ERR_ARG;
    int rc = ODIS_OK;
    if (h->f && std::fclose(h->f) != 0) rc = ODIS_ERR_IO;
    delete h;
    return rc;
}
