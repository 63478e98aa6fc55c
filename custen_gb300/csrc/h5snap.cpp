// HDF5 snapshot files for Cahn-Hilliard state, written and read without the HDF5 library.
//
// The reference solver writes its field every `print` steps with Print_Out
// (cuPentCahnADI/src/cuPentCahnADI.cu:103-140): H5Fcreate with default properties, one two-dimensional
// dataset "/c" of native doubles with dims {nx, ny}, contiguous storage, file name
// "cahn_hilliard_<time %0.10lf>.nc". This file produces and reads that format directly from the
// published HDF5 file-format specification, restricted to what such a file uses:
//
// Writer (the structures the HDF5 library writes for a default-property file):
//   superblock version 0: 8-byte offsets and lengths, group leaf-node K 4, internal-node K 16
//   root group: version-1 object header holding a symbol-table message, which names a version-1
//     B-tree (one leaf) and a local heap of link names (with one free block, as the library leaves)
//   one symbol-table node with up to 8 entries, in strcmp order of their names
//   per dataset: version-1 object header with fill-value (version 1), datatype (IEEE binary64,
//     little-endian), dataspace (version 1) and layout (version 3, contiguous) messages; the data
//     follows the headers, contiguous and row-major
// Reader: superblock version 0 or 1 (a user block before it is skipped); version-1 object headers
//   with continuation messages; group B-trees of any depth; dataspace versions 1 and 2; IEEE
//   floating-point datatypes of 4 or 8 bytes, little-endian; contiguous layouts of versions 1-4.
//   Anything else is refused with an error that names it.
//
// All multi-byte fields are encoded and decoded byte by byte (little-endian), independent of the host.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/custen_gb300.h"

namespace custen {
namespace h5 {

namespace {

thread_local std::string g_error;

int fail(const std::string& msg) {
    g_error = msg;
    return 1;
}

constexpr uint64_t kUndef = ~0ull;           // "undefined address"
constexpr uint64_t kHeapFreeNull = 1;        // end of a local heap's free list (never a valid offset)
constexpr int kLeafK = 4;                    // symbol-table node holds up to 2K entries
constexpr int kInternalK = 16;               // group B-tree node holds up to 2K children
constexpr int kMaxDatasets = 2 * kLeafK;     // one symbol-table node
constexpr size_t kEntrySize = 40;            // symbol-table entry with 8-byte offsets
constexpr size_t kSuperblockSize = 56 + kEntrySize;
constexpr size_t kBtreeSize = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr size_t kSnodSize = 8 + 2 * kLeafK * kEntrySize;
constexpr size_t kRootHeaderSize = 16 + (8 + 16) + 8;   // prefix, symbol-table message, empty NIL message
constexpr size_t kDatasetHeaderSize = 16 + (8 + 8) + (8 + 24) + (8 + 24) + (8 + 24);

size_t round8(size_t v) { return (v + 7) & ~size_t(7); }

struct Out {
    std::vector<uint8_t> b;
    explicit Out(size_t n) : b(n, 0) {}
    void u8(size_t at, uint8_t v) { b[at] = v; }
    void u16(size_t at, uint16_t v) { for (int i = 0; i < 2; ++i) b[at + i] = uint8_t(v >> (8 * i)); }
    void u32(size_t at, uint32_t v) { for (int i = 0; i < 4; ++i) b[at + i] = uint8_t(v >> (8 * i)); }
    void u64(size_t at, uint64_t v) { for (int i = 0; i < 8; ++i) b[at + i] = uint8_t(v >> (8 * i)); }
    void bytes(size_t at, const void* p, size_t n) { std::memcpy(&b[at], p, n); }
};

// Message header of a version-1 object header: type, data size (a multiple of 8), flags.
size_t put_msg(Out& o, size_t at, uint16_t type, uint16_t size, uint8_t flags) {
    o.u16(at, type);
    o.u16(at + 2, size);
    o.u8(at + 4, flags);
    return at + 8;
}

void put_entry(Out& o, size_t at, uint64_t name_off, uint64_t header, uint32_t cache, uint64_t s0, uint64_t s1) {
    o.u64(at, name_off);
    o.u64(at + 8, header);
    o.u32(at + 16, cache);
    o.u64(at + 24, s0);
    o.u64(at + 32, s1);
}

struct In {
    FILE* f = nullptr;
    uint64_t base = 0, size = 0;
    std::string err;
    ~In() { if (f) std::fclose(f); }
    bool read(uint64_t addr, void* dst, size_t n) {
        if (addr > size || n > size - addr) {
            err = "reference past the end of the file";
            return false;
        }
        if (std::fseek(f, (long)(base + addr), SEEK_SET) != 0 || std::fread(dst, 1, n, f) != n) {
            err = "read error";
            return false;
        }
        return true;
    }
    bool bytes(uint64_t addr, std::vector<uint8_t>& v, size_t n) {
        v.resize(n);
        return read(addr, v.data(), n);
    }
};

uint64_t get(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

struct Msg {
    uint16_t type;
    std::vector<uint8_t> data;
};

// Messages of a version-1 object header, following continuation messages (type 0x10).
bool read_messages(In& in, uint64_t addr, std::vector<Msg>& msgs) {
    uint8_t pre[16];
    if (!in.read(addr, pre, 16)) return false;
    if (pre[0] != 1) {
        in.err = pre[0] == 'O' ? "version-2 object headers are not supported" : "bad object header";
        return false;
    }
    const uint32_t nmsgs = (uint32_t)get(pre + 2, 2);
    struct Block { uint64_t addr, len; };
    std::vector<Block> blocks{{addr + 16, get(pre + 8, 4)}};
    for (size_t bi = 0; bi < blocks.size() && msgs.size() < nmsgs; ++bi) {
        if (bi > 64) { in.err = "too many continuation blocks"; return false; }
        std::vector<uint8_t> blk;
        if (!in.bytes(blocks[bi].addr, blk, blocks[bi].len)) return false;
        size_t q = 0;
        while (q + 8 <= blk.size() && msgs.size() < nmsgs) {
            const uint16_t type = (uint16_t)get(&blk[q], 2), sz = (uint16_t)get(&blk[q + 2], 2);
            if (q + 8 + sz > blk.size()) { in.err = "object header message overruns its block"; return false; }
            Msg m{type, std::vector<uint8_t>(blk.begin() + q + 8, blk.begin() + q + 8 + sz)};
            if (type == 0x10) {
                if (sz < 16) { in.err = "short continuation message"; return false; }
                blocks.push_back({get(m.data.data(), 8), get(m.data.data() + 8, 8)});
            }
            msgs.push_back(std::move(m));
            q += 8 + sz;
        }
    }
    return true;
}

bool heap_name(const std::vector<uint8_t>& heap, uint64_t off, std::string& name) {
    if (off >= heap.size()) return false;
    const uint8_t* s = heap.data() + off;
    const void* z = std::memchr(s, 0, heap.size() - off);
    if (!z) return false;
    name.assign(reinterpret_cast<const char*>(s), static_cast<const uint8_t*>(z) - s);
    return true;
}

// Find `name` in a group B-tree; sets *header to its object-header address (kUndef if absent).
bool find_in_btree(In& in, uint64_t node, const std::vector<uint8_t>& heap, const std::string& name,
                   uint64_t* header, int depth) {
    if (depth > 32) { in.err = "group B-tree too deep"; return false; }
    uint8_t hd[24];
    if (!in.read(node, hd, 24)) return false;
    if (std::memcmp(hd, "TREE", 4) != 0 || hd[4] != 0) { in.err = "bad group B-tree node"; return false; }
    const int level = hd[5], used = (int)get(hd + 6, 2);
    std::vector<uint8_t> kc;
    if (!in.bytes(node + 24, kc, (size_t)(2 * used + 1) * 8)) return false;
    for (int i = 0; i < used; ++i) {
        const uint64_t child = get(&kc[(2 * i + 1) * 8], 8);
        if (level > 0) {
            if (!find_in_btree(in, child, heap, name, header, depth + 1)) return false;
        } else {
            uint8_t sh[8];
            if (!in.read(child, sh, 8)) return false;
            if (std::memcmp(sh, "SNOD", 4) != 0) { in.err = "bad symbol-table node"; return false; }
            const int n = (int)get(sh + 6, 2);
            std::vector<uint8_t> ents;
            if (!in.bytes(child + 8, ents, (size_t)n * kEntrySize)) return false;
            for (int e = 0; e < n; ++e) {
                std::string nm;
                if (!heap_name(heap, get(&ents[e * kEntrySize], 8), nm)) { in.err = "bad link name"; return false; }
                if (nm == name) {
                    *header = get(&ents[e * kEntrySize + 8], 8);
                    return true;
                }
            }
        }
        if (*header != kUndef) return true;
    }
    return true;
}

}  // namespace

int write_file(const char* path, int count, const char* const* names, const double* const* data,
               const long long* dims) {
    if (!path || count < 1 || count > kMaxDatasets || !names || !data || !dims)
        return fail("invalid arguments (1 to 8 datasets per file)");
    struct Ds { std::string name; const double* p; uint64_t d0, d1; uint64_t name_off, header, addr; };
    std::vector<Ds> ds;
    for (int i = 0; i < count; ++i) {
        if (!names[i] || !names[i][0] || std::strchr(names[i], '/') || !data[i] || dims[2 * i] < 1 || dims[2 * i + 1] < 1)
            return fail("invalid dataset " + std::to_string(i) + " (name without '/', data, dims >= 1)");
        ds.push_back({names[i], data[i], (uint64_t)dims[2 * i], (uint64_t)dims[2 * i + 1], 0, 0, 0});
    }
    // symbol-table nodes keep their entries in strcmp order of the link names
    for (size_t i = 1; i < ds.size(); ++i)
        for (size_t j = i; j > 0 && std::strcmp(ds[j - 1].name.c_str(), ds[j].name.c_str()) > 0; --j) std::swap(ds[j - 1], ds[j]);
    for (size_t i = 1; i < ds.size(); ++i)
        if (ds[i].name == ds[i - 1].name) return fail("duplicate dataset name " + ds[i].name);

    // local heap data: the empty name at 0, the link names (8-byte padded), then one free block
    size_t used = 8;
    for (auto& d : ds) {
        d.name_off = used;
        used += round8(d.name.size() + 1);
    }
    const size_t heap_free = 16 + 8 * kMaxDatasets;
    const size_t heap_size = used + heap_free;

    const size_t a_root = kSuperblockSize;
    const size_t a_heap = a_root + kRootHeaderSize;
    const size_t a_heap_data = a_heap + 32;
    const size_t a_btree = a_heap_data + heap_size;
    const size_t a_snod = a_btree + kBtreeSize;
    size_t at = a_snod + kSnodSize;
    for (auto& d : ds) {
        d.header = at;
        at += kDatasetHeaderSize;
    }
    const size_t meta = at;
    uint64_t eof = meta;
    for (auto& d : ds) {
        d.addr = eof;
        eof += d.d0 * d.d1 * 8;
    }

    Out o(meta);
    // superblock
    o.bytes(0, "\x89HDF\r\n\x1a\n", 8);
    o.u8(13, 8);                 // size of offsets (versions and reserved bytes 8..12 and 15 are zero)
    o.u8(14, 8);                 // size of lengths
    o.u16(16, kLeafK);
    o.u16(18, kInternalK);
    o.u32(20, 0);                // file consistency flags
    o.u64(24, 0);                // base address
    o.u64(32, kUndef);           // free-space info
    o.u64(40, eof);              // end-of-file address
    o.u64(48, kUndef);           // driver information block
    put_entry(o, 56, 0, a_root, 1, a_btree, a_heap);   // root group, B-tree and heap cached
    // root group object header: symbol-table message, then an empty NIL message
    o.u8(a_root, 1);
    o.u16(a_root + 2, 2);
    o.u32(a_root + 4, 1);
    o.u32(a_root + 8, (uint32_t)(kRootHeaderSize - 16));
    size_t q = put_msg(o, a_root + 16, 0x0011, 16, 1);
    o.u64(q, a_btree);
    o.u64(q + 8, a_heap);
    put_msg(o, q + 16, 0x0000, 0, 0);
    // local heap
    o.bytes(a_heap, "HEAP", 4);
    o.u64(a_heap + 8, heap_size);
    o.u64(a_heap + 16, used);                       // head of the free list
    o.u64(a_heap + 24, a_heap_data);
    for (auto& d : ds) o.bytes(a_heap_data + d.name_off, d.name.c_str(), d.name.size());
    o.u64(a_heap_data + used, kHeapFreeNull);       // the free block: next, size
    o.u64(a_heap_data + used + 8, heap_free);
    // group B-tree: one leaf pointing at the symbol-table node; key 0 = "", key 1 = the last name
    o.bytes(a_btree, "TREE", 4);
    o.u8(a_btree + 4, 0);
    o.u8(a_btree + 5, 0);
    o.u16(a_btree + 6, 1);
    o.u64(a_btree + 8, kUndef);
    o.u64(a_btree + 16, kUndef);
    o.u64(a_btree + 24, 0);
    o.u64(a_btree + 32, a_snod);
    o.u64(a_btree + 40, ds.back().name_off);
    // symbol-table node
    o.bytes(a_snod, "SNOD", 4);
    o.u8(a_snod + 4, 1);
    o.u16(a_snod + 6, (uint16_t)ds.size());
    for (size_t i = 0; i < ds.size(); ++i) put_entry(o, a_snod + 8 + i * kEntrySize, ds[i].name_off, ds[i].header, 0, 0, 0);
    // dataset object headers
    for (auto& d : ds) {
        const size_t h = d.header;
        o.u8(h, 1);
        o.u16(h + 2, 4);
        o.u32(h + 4, 1);
        o.u32(h + 8, (uint32_t)(kDatasetHeaderSize - 16));
        // fill value, version 1: allocation late, written if set, defined with size 0 (the default)
        q = put_msg(o, h + 16, 0x0005, 8, 1);
        o.u8(q, 1); o.u8(q + 1, 2); o.u8(q + 2, 2); o.u8(q + 3, 1);
        // datatype: version 1, class 1 (floating point); bit field: little-endian, implied mantissa
        // MSB, sign at bit 63; 8 bytes; offset 0, precision 64, exponent at 52 of 11 bits, mantissa at
        // 0 of 52 bits, exponent bias 1023
        q = put_msg(o, q + 8, 0x0003, 24, 1);
        o.u8(q, 0x11); o.u8(q + 1, 0x20); o.u8(q + 2, 63); o.u8(q + 3, 0);
        o.u32(q + 4, 8);
        o.u16(q + 8, 0); o.u16(q + 10, 64);
        o.u8(q + 12, 52); o.u8(q + 13, 11); o.u8(q + 14, 0); o.u8(q + 15, 52);
        o.u32(q + 16, 1023);
        // dataspace, version 1: rank 2, no maximum dims
        q = put_msg(o, q + 24, 0x0001, 24, 0);
        o.u8(q, 1); o.u8(q + 1, 2);
        o.u64(q + 8, d.d0);
        o.u64(q + 16, d.d1);
        // layout, version 3: contiguous, address and size
        q = put_msg(o, q + 24, 0x0008, 24, 1);
        o.u8(q, 3); o.u8(q + 1, 1);
        o.u64(q + 2, d.addr);
        o.u64(q + 10, d.d0 * d.d1 * 8);
    }

    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(std::string("cannot create ") + path + ": " + std::strerror(errno));
    bool ok = std::fwrite(o.b.data(), 1, o.b.size(), f) == o.b.size();
    std::vector<uint8_t> buf;
    for (auto& d : ds) {
        const size_t n = d.d0 * d.d1;
        const size_t chunk = 1 << 16;
        buf.resize(chunk * 8);
        for (size_t i = 0; ok && i < n; i += chunk) {
            const size_t m = n - i < chunk ? n - i : chunk;
            for (size_t k = 0; k < m; ++k) {
                uint64_t bits;
                std::memcpy(&bits, d.p + i + k, 8);
                for (int j = 0; j < 8; ++j) buf[8 * k + j] = uint8_t(bits >> (8 * j));
            }
            ok = std::fwrite(buf.data(), 1, m * 8, f) == m * 8;
        }
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return fail(std::string("write error on ") + path);
    return 0;
}

int read_dataset(const char* path, const char* name, double* out, long long capacity, long long* dims) {
    if (!path || !name || !dims) return fail("invalid arguments");
    In in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return fail(std::string("cannot open ") + path + ": " + std::strerror(errno));
    std::fseek(in.f, 0, SEEK_END);
    const uint64_t fsize = (uint64_t)std::ftell(in.f);
    // the superblock sits at 0 or after a user block of 512, 1024, 2048, ... bytes
    uint64_t sb = kUndef;
    for (uint64_t off = 0; off + 8 <= fsize; off = off ? off * 2 : 512) {
        uint8_t sig[8];
        std::fseek(in.f, (long)off, SEEK_SET);
        if (std::fread(sig, 1, 8, in.f) == 8 && std::memcmp(sig, "\x89HDF\r\n\x1a\n", 8) == 0) { sb = off; break; }
    }
    if (sb == kUndef) return fail(std::string(path) + ": not an HDF5 file");
    in.size = fsize;
    uint8_t s[128];
    if (!in.read(sb, s, 24)) return fail(in.err);
    const int version = s[8];
    if (version > 1) return fail(std::string(path) + ": superblock version " + std::to_string(version) + " is not supported");
    if (s[13] != 8 || s[14] != 8) return fail(std::string(path) + ": only 8-byte offsets and lengths are supported");
    const size_t rest = version == 1 ? 4 : 0;      // version 1 adds indexed-storage K and a reserved field
    if (!in.read(sb + 24 + rest, s + 24, 32 + kEntrySize)) return fail(in.err);
    in.base = get(s + 24, 8);
    in.size = fsize - in.base;
    const uint64_t root = get(s + 56 + 8, 8);

    std::vector<Msg> msgs;
    if (!read_messages(in, root, msgs)) return fail(std::string(path) + ": root group: " + in.err);
    uint64_t btree = kUndef, heap_addr = kUndef;
    for (auto& m : msgs)
        if (m.type == 0x0011 && m.data.size() >= 16) {
            btree = get(m.data.data(), 8);
            heap_addr = get(m.data.data() + 8, 8);
        }
    if (btree == kUndef) return fail(std::string(path) + ": the root group has no symbol table (new-style groups are not supported)");
    uint8_t hh[32];
    if (!in.read(heap_addr, hh, 32) || std::memcmp(hh, "HEAP", 4) != 0) return fail(std::string(path) + ": bad local heap");
    std::vector<uint8_t> heap;
    if (!in.bytes(get(hh + 24, 8), heap, get(hh + 8, 8))) return fail(std::string(path) + ": local heap: " + in.err);
    uint64_t header = kUndef;
    if (!find_in_btree(in, btree, heap, name, &header, 0)) return fail(std::string(path) + ": " + in.err);
    if (header == kUndef) return fail(std::string(path) + ": no dataset named " + name);

    msgs.clear();
    if (!read_messages(in, header, msgs)) return fail(std::string(path) + ": dataset " + name + ": " + in.err);
    std::vector<uint64_t> shape;
    int elem = 0;
    uint64_t addr = kUndef, bytes = 0;
    bool have_space = false, have_type = false, have_layout = false;
    for (auto& m : msgs) {
        const uint8_t* p = m.data.data();
        const size_t n = m.data.size();
        if (m.type == 0x0001 && n >= 8) {           // dataspace
            const int v = p[0], rank = p[1];
            const size_t d0 = v == 1 ? 8 : 4;
            if ((v != 1 && v != 2) || n < d0 + 8 * (size_t)rank) return fail("dataset " + std::string(name) + ": unsupported dataspace");
            for (int r = 0; r < rank; ++r) shape.push_back(get(p + d0 + 8 * r, 8));
            have_space = true;
        } else if (m.type == 0x0003 && n >= 8) {    // datatype
            const int cls = p[0] & 0x0f;
            elem = (int)get(p + 4, 4);
            if (cls != 1 || (p[1] & 1) || (elem != 8 && elem != 4))
                return fail("dataset " + std::string(name) + ": only little-endian IEEE float32/float64 data is supported");
            have_type = true;
        } else if (m.type == 0x0008 && n >= 2) {    // layout
            const int v = p[0];
            if (v == 1 || v == 2) {
                if (n < 16 || p[2] != 1) return fail("dataset " + std::string(name) + ": only contiguous storage is supported");
                addr = get(p + 8, 8);
            } else if (v == 3 || v == 4) {
                if (n < 18 || p[1] != 1) return fail("dataset " + std::string(name) + ": only contiguous storage is supported");
                addr = get(p + 2, 8);
                bytes = get(p + 10, 8);
            } else {
                return fail("dataset " + std::string(name) + ": layout message version " + std::to_string(v) + " is not supported");
            }
            have_layout = true;
        } else if (m.type == 0x000B || m.type == 0x0016) {
            return fail("dataset " + std::string(name) + ": filtered (compressed) data is not supported");
        }
    }
    if (!have_space || !have_type || !have_layout) return fail("dataset " + std::string(name) + ": incomplete object header");
    if (shape.size() > 2) return fail("dataset " + std::string(name) + ": rank above 2 is not supported");
    uint64_t count = 1;
    for (uint64_t d : shape) count *= d;
    dims[0] = shape.size() > 0 ? (long long)shape[0] : 1;
    dims[1] = shape.size() > 1 ? (long long)shape[1] : 1;
    if (!out) return 0;
    if ((long long)count > capacity) return fail("dataset " + std::string(name) + ": output buffer too small");
    if (addr == kUndef) {                           // storage never written: the default fill value
        for (uint64_t i = 0; i < count; ++i) out[i] = 0.0;
        return 0;
    }
    if (bytes && bytes < count * elem) return fail("dataset " + std::string(name) + ": storage smaller than its dataspace");
    std::vector<uint8_t> raw;
    if (!in.bytes(addr, raw, count * elem)) return fail("dataset " + std::string(name) + ": " + in.err);
    for (uint64_t i = 0; i < count; ++i) {
        if (elem == 8) {
            const uint64_t bits = get(&raw[8 * i], 8);
            std::memcpy(&out[i], &bits, 8);
        } else {
            const uint32_t bits = (uint32_t)get(&raw[4 * i], 4);
            float fv;
            std::memcpy(&fv, &bits, 4);
            out[i] = fv;
        }
    }
    return 0;
}

}  // namespace h5
}  // namespace custen

extern "C" {

int custen_h5_write(const char* path, int count, const char* const* names, const double* const* data,
                    const long long* dims) {
    return custen::h5::write_file(path, count, names, data, dims);
}

int custen_h5_read(const char* path, const char* name, double* out, long long capacity, long long* dims) {
    return custen::h5::read_dataset(path, name, out, capacity, dims);
}

const char* custen_h5_last_error(void) { return custen::h5::g_error.c_str(); }

}  // extern "C"
