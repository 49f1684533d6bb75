// HDF5 writer: superblock 0, version-1 object headers, one symbol-table root group, contiguous
// FP64 datasets and scalar-like (one-element) attributes. Structure sizes and field orders
// follow the HDF5 file format specification (superblock, object header prefix and messages:
// dataspace 0x1, datatype 0x3, fill value 0x5, layout 0x8, attribute 0xC, symbol table 0x11;
// version-1 B-tree "TREE", symbol-table node "SNOD", local heap "HEAP").
#include "h5write.hpp"

#include <algorithm>
#include <cstring>
#include <fstream>

#include "common.hpp"

namespace tdg {

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 16;      // a symbol-table node holds 2K = 32 entries
constexpr int kInternalK = 16;  // group B-tree nodes hold up to 2K children
constexpr size_t kBtreeBytes = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr size_t kSnodBytes = 8 + 2 * kLeafK * 40;

size_t pad8(size_t x) { return (x + 7) & ~size_t(7); }

struct Bytes {
    std::vector<uint8_t> b;
    void u8(uint64_t v) { b.push_back((uint8_t)v); }
    void u16(uint64_t v) { for (int i = 0; i < 2; ++i) u8(v >> (8 * i)); }
    void u32(uint64_t v) { for (int i = 0; i < 4; ++i) u8(v >> (8 * i)); }
    void u64(uint64_t v) { for (int i = 0; i < 8; ++i) u8(v >> (8 * i)); }
    void raw(const void *p, size_t n) {
        const uint8_t *c = static_cast<const uint8_t *>(p);
        b.insert(b.end(), c, c + n);
    }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad_to(size_t mult) { zeros((mult - b.size() % mult) % mult); }
    size_t size() const { return b.size(); }
};

// Datatype messages (version 1): signed 32-bit little-endian integer, IEEE little-endian
// double, fixed-length null-padded ASCII string.
Bytes dt_int32() {
    Bytes d;
    d.u8(0x10);
    d.u8(0x08);
    d.u8(0);
    d.u8(0);
    d.u32(4);
    d.u16(0);
    d.u16(32);
    return d;
}
Bytes dt_double() {
    Bytes d;
    d.u8(0x11);
    d.u8(0x20);
    d.u8(63);
    d.u8(0);
    d.u32(8);
    d.u16(0);
    d.u16(64);
    d.u8(52);
    d.u8(11);
    d.u8(0);
    d.u8(52);
    d.u32(1023);
    return d;
}
Bytes dt_string(size_t len) {
    Bytes d;
    d.u8(0x13);
    d.u8(0x01);
    d.u8(0);
    d.u8(0);
    d.u32((uint32_t)len);
    return d;
}
// Simple dataspace (version 1), no maximum dimensions.
Bytes dataspace(const std::vector<uint64_t> &dims) {
    Bytes d;
    d.u8(1);
    d.u8(dims.size());
    d.u8(0);
    d.u8(0);
    d.u32(0);
    for (uint64_t x : dims) d.u64(x);
    return d;
}

// One message of a version-1 object header: type, size, flags, reserved, data padded to 8.
void message(Bytes &oh, int type, const Bytes &data) {
    const size_t sz = pad8(data.size());
    oh.u16(type);
    oh.u16(sz);
    oh.u8(0);
    oh.zeros(3);
    oh.raw(data.b.data(), data.size());
    oh.zeros(sz - data.size());
}

template <typename A>
Bytes attribute(const A &a) {
    Bytes dt, value;
    if (a.kind == 0) {
        dt = dt_int32();
        value.u32((uint32_t)a.i);
    } else if (a.kind == 1) {
        dt = dt_double();
        value.raw(&a.d, 8);
    } else {
        const size_t len = std::max<size_t>(1, a.s.size());
        dt = dt_string(len);
        value.raw(a.s.data(), a.s.size());
        value.zeros(len - a.s.size());
    }
    const Bytes ds = dataspace({1});
    Bytes m;
    m.u8(1);
    m.u8(0);
    m.u16(a.name.size() + 1);
    m.u16(dt.size());
    m.u16(ds.size());
    m.raw(a.name.data(), a.name.size());
    m.u8(0);
    m.pad_to(8);
    m.raw(dt.b.data(), dt.size());
    m.pad_to(8);
    m.raw(ds.b.data(), ds.size());
    m.pad_to(8);
    m.raw(value.b.data(), value.size());
    return m;
}

// Version-1 object header from its messages (prefix of 12 bytes aligned to 16).
Bytes object_header(const std::vector<std::pair<int, Bytes>> &msgs) {
    Bytes body;
    for (const auto &m : msgs) message(body, m.first, m.second);
    Bytes oh;
    oh.u8(1);
    oh.u8(0);
    oh.u16(msgs.size());
    oh.u32(1);
    oh.u32(body.size());
    oh.u32(0);
    oh.raw(body.b.data(), body.size());
    return oh;
}

}  // namespace

void H5Writer::attr_int(const std::string &name, int32_t v) { root_attrs_.push_back({name, 0, v, 0.0, ""}); }
void H5Writer::attr_double(const std::string &name, double v) { root_attrs_.push_back({name, 1, 0, v, ""}); }
void H5Writer::attr_string(const std::string &name, const std::string &v) {
    root_attrs_.push_back({name, 2, 0, 0.0, v});
}
void H5Writer::dataset(const std::string &name, const std::vector<uint64_t> &dims, std::vector<double> data,
                       const std::string &unit, const std::string &dimensions) {
    Dset d{name, dims, std::move(data), {}};
    if (!unit.empty()) d.attrs.push_back({"unit", 2, 0, 0.0, unit});
    if (!dimensions.empty()) d.attrs.push_back({"dimensions", 2, 0, 0.0, dimensions});
    dsets_.push_back(std::move(d));
}

int H5Writer::write(const std::string &path) const {
    if (dsets_.size() > (size_t)(2 * kLeafK))
        return set_error(kErrParam, "HDF5 writer: more datasets than one symbol-table node holds");
    for (const auto &d : dsets_) {
        uint64_t cnt = 1;
        for (uint64_t x : d.dims) cnt *= x;
        if (cnt != d.data.size()) return set_error(kErrParam, "HDF5 writer: dataset size does not match its dims");
    }
    std::vector<const Dset *> order;
    for (const auto &d : dsets_) order.push_back(&d);
    std::sort(order.begin(), order.end(), [](const Dset *a, const Dset *b) { return a->name < b->name; });
    // local heap data segment: "" at offset 0, the names, then one free block (next = 1,
    // the format's "no next block", and its size)
    Bytes heap;
    heap.zeros(8);
    std::vector<uint64_t> name_off;
    for (const Dset *d : order) {
        name_off.push_back(heap.size());
        heap.raw(d->name.data(), d->name.size());
        heap.u8(0);
        heap.pad_to(8);
    }
    const uint64_t free_off = heap.size();
    heap.u64(1);
    heap.u64(16);
    // addresses
    const uint64_t a_sb = 0, a_root = 96;
    std::vector<std::pair<int, Bytes>> root_msgs;
    Bytes symtab;
    symtab.zeros(16);  // patched below
    root_msgs.push_back({0x11, symtab});
    for (const auto &a : root_attrs_) root_msgs.push_back({0x0C, attribute(a)});
    const size_t root_size = object_header(root_msgs).size();
    const uint64_t a_btree = pad8(a_root + root_size);
    const uint64_t a_heap = a_btree + kBtreeBytes;
    const uint64_t a_heapdata = a_heap + 32;
    const uint64_t a_snod = pad8(a_heapdata + heap.size());
    uint64_t p = a_snod + kSnodBytes;
    // dataset object headers: sizes do not depend on the data address, so build them twice
    auto dset_header = [&](const Dset *d, uint64_t data_addr) {
        std::vector<std::pair<int, Bytes>> m;
        m.push_back({0x01, dataspace(d->dims)});
        m.push_back({0x03, dt_double()});
        Bytes fill;
        fill.u8(2);  // version 2: allocated early, written if set, no fill value defined
        fill.u8(1);
        fill.u8(2);
        fill.u8(0);
        m.push_back({0x05, fill});
        Bytes lay;
        lay.u8(3);
        lay.u8(1);  // contiguous
        lay.u64(data_addr);
        lay.u64(8 * d->data.size());
        m.push_back({0x08, lay});
        for (const auto &a : d->attrs) m.push_back({0x0C, attribute(a)});
        return object_header(m);
    };
    std::vector<uint64_t> a_oh(order.size()), a_data(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
        a_oh[i] = p;
        p = pad8(p + dset_header(order[i], 0).size());
    }
    for (size_t i = 0; i < order.size(); ++i) {
        a_data[i] = p;
        p = pad8(p + 8 * order[i]->data.size());
    }
    const uint64_t eof = p;
    // serialise
    Bytes f;
    f.raw("\x89HDF\r\n\x1a\n", 8);
    f.u8(0);
    f.u8(0);
    f.u8(0);
    f.u8(0);
    f.u8(0);
    f.u8(8);
    f.u8(8);
    f.u8(0);
    f.u16(kLeafK);
    f.u16(kInternalK);
    f.u32(0);
    f.u64(0);
    f.u64(kUndef);
    f.u64(eof);
    f.u64(kUndef);
    f.u64(0);       // root entry: link name offset
    f.u64(a_root);  // object header
    f.u32(1);       // cache type 1: B-tree and heap addresses in the scratch pad
    f.u32(0);
    f.u64(a_btree);
    f.u64(a_heap);
    (void)a_sb;
    Bytes st;
    st.u64(a_btree);
    st.u64(a_heap);
    root_msgs[0].second = st;
    const Bytes root = object_header(root_msgs);
    f.raw(root.b.data(), root.size());
    f.zeros(a_btree - f.size());
    // group B-tree: one leaf node with one symbol-table node
    f.raw("TREE", 4);
    f.u8(0);
    f.u8(0);
    f.u16(1);
    f.u64(kUndef);
    f.u64(kUndef);
    f.u64(0);
    f.u64(a_snod);
    f.u64(name_off.empty() ? 0 : name_off.back());
    f.zeros(a_heap - f.size());
    f.raw("HEAP", 4);
    f.u8(0);
    f.zeros(3);
    f.u64(heap.size());
    f.u64(free_off);
    f.u64(a_heapdata);
    f.raw(heap.b.data(), heap.size());
    f.zeros(a_snod - f.size());
    f.raw("SNOD", 4);
    f.u8(1);
    f.u8(0);
    f.u16(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
        f.u64(name_off[i]);
        f.u64(a_oh[i]);
        f.u32(0);
        f.u32(0);
        f.zeros(16);
    }
    f.zeros(a_snod + kSnodBytes - f.size());
    for (size_t i = 0; i < order.size(); ++i) {
        f.zeros(a_oh[i] - f.size());
        const Bytes oh = dset_header(order[i], a_data[i]);
        f.raw(oh.b.data(), oh.size());
    }
    for (size_t i = 0; i < order.size(); ++i) {
        f.zeros(a_data[i] - f.size());
        f.raw(order[i]->data.data(), 8 * order[i]->data.size());
    }
    f.zeros(eof - f.size());
    std::ofstream out(path, std::ios::binary);
    if (!out) return set_error(kErrIo, "cannot write " + path);
    out.write(reinterpret_cast<const char *>(f.b.data()), (std::streamsize)f.size());
    if (!out) return set_error(kErrIo, "write failed: " + path);
    return kOk;
}

}  // namespace tdg
