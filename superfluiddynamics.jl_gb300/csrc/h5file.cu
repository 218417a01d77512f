// HDF5 checkpoint files in the layout of the reference's WriterSave
// (src/IO/Writers.jl:42-96 write!, :116-137 read!): one file
// "<prefix>-<istep>.h5" per checkpoint holding two float64 datasets, "re" and
// "im", with Re psi and Im psi.  Julia hands HDF5 its column-major
// (nx, ny[, nz]) arrays with the dimension list reversed (HDF5 dataspaces are
// row-major), so the dataspace is (nz, ny, nx) / (ny, nx) over the same
// bytes: x fastest, the order of the C ABI's field buffers.
//
// No HDF5 library is linked.  The writer emits the format's classic
// structures itself: a version 0 superblock, version 1 object headers, a
// symbol-table root group (one local heap, one v1 B-tree leaf, one symbol
// table node), contiguous storage of little-endian IEEE doubles.  The reader
// accepts that subset of the format as the HDF5 library writes it
// (superblock 0 or 1 after an optional user block, v1 object headers with
// continuation blocks, symbol-table groups with B-trees of any depth,
// dataspace messages 1 and 2, layout messages 1-3 with contiguous or compact
// storage, IEEE float32/float64 in either byte order) and reports anything
// else (v2 object headers, link-message groups, chunked or filtered storage)
// as an error instead of guessing.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "ctx.cuh"
#include "gpss.h"

namespace {

constexpr uint64_t kUndef = ~0ull;  // the format's undefined address
constexpr int kLeafK = 4;           // group leaf node K: 2K entries per symbol table node
constexpr int kNodeK = 16;          // group internal node K: 2K children per B-tree node

bool host_is_le()
{
    const uint32_t one = 1;
    uint8_t b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// ------------------------------------------------------------------ writer --
struct Out {
    std::vector<uint8_t> b;
    void u8(unsigned v) { b.push_back((uint8_t)(v & 0xffu)); }
    void u16(unsigned v) { u8(v); u8(v >> 8); }
    void u32(uint32_t v)
    {
        for (int i = 0; i < 4; i++) u8(v >> (8 * i));
    }
    void u64(uint64_t v)
    {
        for (int i = 0; i < 8; i++) u8((unsigned)(v >> (8 * i)));
    }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8()
    {
        while (b.size() % 8) u8(0);
    }
    void put64(size_t at, uint64_t v)
    {
        for (int i = 0; i < 8; i++) b[at + i] = (uint8_t)(v >> (8 * i));
    }
    void put32(size_t at, uint32_t v)
    {
        for (int i = 0; i < 4; i++) b[at + i] = (uint8_t)(v >> (8 * i));
    }
};

// One object header message of a version 1 header: type, data size (padded
// to 8 bytes), flags, 3 reserved bytes, then the data.
template <typename F> void message(Out &o, unsigned type, unsigned flags, F body)
{
    const size_t head = o.b.size();
    o.u16(type);
    o.u16(0);  // size, patched below
    o.u8(flags);
    o.zeros(3);
    const size_t start = o.b.size();
    body();
    o.pad8();
    const size_t n = o.b.size() - start;
    o.b[head + 2] = (uint8_t)(n & 0xff);
    o.b[head + 3] = (uint8_t)(n >> 8);
}

struct Dataset {
    std::string name;
    const double *data;
};

// A file holding float64 datasets of one shape (dims slowest first) in the
// root group.  Names must be distinct; at most 2 * kLeafK of them.
int write_file(const char *path, int rank, const uint64_t *dims, std::vector<Dataset> sets, std::string &err)
{
    if (sets.empty() || (int)sets.size() > 2 * kLeafK) {
        err = "h5: 1 to 8 datasets per file";
        return GPSS_EINVAL;
    }
    std::sort(sets.begin(), sets.end(), [](const Dataset &a, const Dataset &b) { return a.name < b.name; });
    uint64_t count = 1;
    for (int i = 0; i < rank; i++) count *= dims[i];
    const uint64_t nbytes = count * 8;

    Out o;
    // superblock, version 0 (96 bytes with 8-byte offsets and lengths)
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    for (uint8_t c : sig) o.u8(c);
    o.u8(0);  // superblock version
    o.u8(0);  // free-space storage version
    o.u8(0);  // root group symbol table entry version
    o.u8(0);
    o.u8(0);  // shared header message format version
    o.u8(8);  // size of offsets
    o.u8(8);  // size of lengths
    o.u8(0);
    o.u16(kLeafK);
    o.u16(kNodeK);
    o.u32(0);  // file consistency flags
    o.u64(0);  // base address
    o.u64(kUndef);  // free-space info
    const size_t at_eof = o.b.size();
    o.u64(0);  // end of file address, patched
    o.u64(kUndef);  // driver information block
    // root group symbol table entry: link name offset, object header, cache
    // type 1 (scratch pad holds the B-tree and heap addresses)
    o.u64(0);
    const size_t at_root_oh = o.b.size();
    o.u64(0);
    o.u32(1);
    o.u32(0);
    const size_t at_root_scratch = o.b.size();
    o.u64(0);
    o.u64(0);

    // root group object header: one symbol table message
    o.pad8();
    const uint64_t root_oh = o.b.size();
    o.u8(1);  // version
    o.u8(0);
    o.u16(1);  // messages
    o.u32(1);  // reference count
    const size_t at_root_size = o.b.size();
    o.u32(0);  // header data size, patched
    o.u32(0);  // alignment padding of the version 1 prefix
    const size_t root_msgs = o.b.size();
    size_t at_symtab = 0;
    message(o, 0x0011, 1, [&] {
        at_symtab = o.b.size();
        o.u64(0);  // B-tree
        o.u64(0);  // local heap
    });
    o.put32(at_root_size, (uint32_t)(o.b.size() - root_msgs));

    // local heap: "" at offset 0, then the names (each padded to 8 bytes),
    // then one free block (next = 1: end of the free list)
    std::vector<uint64_t> name_off;
    Out heap;
    heap.zeros(8);
    for (const Dataset &s : sets) {
        name_off.push_back(heap.b.size());
        for (char ch : s.name) heap.u8((unsigned char)ch);
        heap.u8(0);
        heap.pad8();
    }
    const uint64_t free_off = heap.b.size();
    heap.u64(1);
    heap.u64(64);
    heap.zeros(64 - 16);
    const uint64_t heap_addr = o.b.size();
    o.b.insert(o.b.end(), {'H', 'E', 'A', 'P'});
    o.u8(0);
    o.zeros(3);
    o.u64(heap.b.size());
    o.u64(free_off);
    o.u64(heap_addr + 32);
    o.b.insert(o.b.end(), heap.b.begin(), heap.b.end());

    // B-tree (group nodes, one leaf): key0, child0, key1; allocated at the
    // full node size the reader computes from K
    o.pad8();
    const uint64_t btree = o.b.size();
    o.b.insert(o.b.end(), {'T', 'R', 'E', 'E'});
    o.u8(0);  // group node
    o.u8(0);  // level 0
    o.u16(1);  // entries used
    o.u64(kUndef);
    o.u64(kUndef);
    o.u64(0);  // key 0: the empty name
    const size_t at_child = o.b.size();
    o.u64(0);  // child 0: the symbol table node, patched
    o.u64(name_off.back());  // key 1: the largest name in child 0
    o.zeros(24 + (size_t)(2 * kNodeK) * 8 + (size_t)(2 * kNodeK + 1) * 8 - (o.b.size() - btree));

    // symbol table node, allocated for 2 * kLeafK entries
    const uint64_t snod = o.b.size();
    o.put64(at_child, snod);
    o.b.insert(o.b.end(), {'S', 'N', 'O', 'D'});
    o.u8(1);  // version
    o.u8(0);
    o.u16((unsigned)sets.size());
    std::vector<size_t> at_entry_oh;
    for (size_t i = 0; i < sets.size(); i++) {
        o.u64(name_off[i]);
        at_entry_oh.push_back(o.b.size());
        o.u64(0);  // object header, patched
        o.u32(0);  // cache type 0
        o.u32(0);
        o.zeros(16);
    }
    o.zeros(8 + (size_t)(2 * kLeafK) * 40 - (o.b.size() - snod));

    // dataset object headers: dataspace, datatype, fill value, layout
    std::vector<size_t> at_data;
    for (size_t i = 0; i < sets.size(); i++) {
        o.pad8();
        o.put64(at_entry_oh[i], o.b.size());
        o.u8(1);
        o.u8(0);
        o.u16(4);
        o.u32(1);
        const size_t at_size = o.b.size();
        o.u32(0);
        o.u32(0);
        const size_t msgs = o.b.size();
        message(o, 0x0001, 0, [&] {  // dataspace, version 1, no maximum dims
            o.u8(1);
            o.u8((unsigned)rank);
            o.u8(0);
            o.u8(0);
            o.u32(0);
            for (int d = 0; d < rank; d++) o.u64(dims[d]);
        });
        message(o, 0x0003, 1, [&] {  // IEEE float64, little-endian
            o.u8(0x11);  // version 1, class 1 (floating point)
            o.u8(0x20);  // byte order LE, no padding, mantissa normalisation 2 (implied msb)
            o.u8(63);    // sign bit position
            o.u8(0);
            o.u32(8);
            o.u16(0);   // bit offset
            o.u16(64);  // precision
            o.u8(52);   // exponent location
            o.u8(11);   // exponent size
            o.u8(0);    // mantissa location
            o.u8(52);   // mantissa size
            o.u32(1023);
        });
        message(o, 0x0005, 1, [&] {  // fill value: version 1, late allocation, write if set, default value
            o.u8(1);
            o.u8(2);
            o.u8(2);
            o.u8(1);
            o.u32(0);
        });
        message(o, 0x0008, 0, [&] {  // layout version 3, contiguous
            o.u8(3);
            o.u8(1);
            at_data.push_back(o.b.size());
            o.u64(0);  // address, patched
            o.u64(nbytes);
        });
        o.put32(at_size, (uint32_t)(o.b.size() - msgs));
    }
    o.pad8();
    uint64_t data_addr = o.b.size();
    for (size_t i = 0; i < sets.size(); i++) {
        o.put64(at_data[i], data_addr);
        data_addr += nbytes;
    }
    o.put64(at_eof, data_addr);
    o.put64(at_root_oh, root_oh);
    o.put64(at_root_scratch, btree);
    o.put64(at_root_scratch + 8, heap_addr);
    o.put64(at_symtab, btree);
    o.put64(at_symtab + 8, heap_addr);

    FILE *fp = std::fopen(path, "wb");
    if (!fp) {
        err = std::string("h5: cannot create ") + path + ": " + std::strerror(errno);
        return GPSS_EIO;
    }
    bool ok = std::fwrite(o.b.data(), 1, o.b.size(), fp) == o.b.size();
    // raw data: little-endian IEEE doubles, written in blocks
    std::vector<uint8_t> blk;
    for (size_t i = 0; ok && i < sets.size(); i++) {
        const double *src = sets[i].data;
        const uint64_t step = 1 << 16;
        for (uint64_t e = 0; ok && e < count; e += step) {
            const uint64_t m = std::min<uint64_t>(step, count - e);
            if (host_is_le()) {  // the doubles are already the file's bytes
                ok = std::fwrite(src + e, 8, m, fp) == m;
                continue;
            }
            blk.resize(m * 8);
            for (uint64_t j = 0; j < m; j++) {
                uint64_t bits;
                std::memcpy(&bits, &src[e + j], 8);
                for (int k = 0; k < 8; k++) blk[j * 8 + k] = (uint8_t)(bits >> (8 * k));
            }
            ok = std::fwrite(blk.data(), 1, blk.size(), fp) == blk.size();
        }
    }
    if (std::fclose(fp) != 0) ok = false;
    if (!ok) {
        err = std::string("h5: write failed: ") + path;
        return GPSS_EIO;
    }
    return GPSS_OK;
}

// ------------------------------------------------------------------ reader --
struct Message {
    unsigned type;
    std::vector<uint8_t> data;
};

uint64_t le(const uint8_t *p, int n)
{
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; i--) v = (v << 8) | p[i];
    return v;
}

struct In {
    FILE *fp = nullptr;
    uint64_t base = 0, size = 0;
    std::string err;
    ~In()
    {
        if (fp) std::fclose(fp);
    }
    bool fail(const std::string &m)
    {
        if (err.empty()) err = "h5: " + m;
        return false;
    }
    // bytes at a file-relative address (the superblock's base applied)
    bool at(uint64_t addr, void *dst, size_t n)
    {
        const uint64_t a = base + addr;
        if (addr == kUndef || a < addr || a > size || n > size - a) return fail("address out of the file");
        if (std::fseek(fp, (long)a, SEEK_SET) != 0 || std::fread(dst, 1, n, fp) != n) return fail("read failed");
        return true;
    }
    bool open(const char *path)
    {
        fp = std::fopen(path, "rb");
        if (!fp) return fail(std::string("cannot open ") + path + ": " + std::strerror(errno));
        if (std::fseek(fp, 0, SEEK_END) != 0) return fail("cannot size the file");
        const long s = std::ftell(fp);
        if (s < 0) return fail("cannot size the file");
        size = (uint64_t)s;
        return true;
    }
};

struct Superblock {
    uint64_t root_oh = 0;
};

bool read_superblock(In &in, Superblock &sb)
{
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    // the signature sits at 0, 512, 1024, 2048, ... (after a user block)
    for (uint64_t off = 0; off + 8 <= in.size; off = off ? off * 2 : 512) {
        uint8_t s[8];
        in.base = 0;
        if (!in.at(off, s, 8)) return false;
        if (std::memcmp(s, sig, 8) != 0) continue;
        uint8_t h[28];
        if (!in.at(off + 8, h, sizeof h)) return false;
        const int ver = h[0];
        if (ver > 1) return in.fail("superblock version " + std::to_string(ver) + " (only 0 and 1 are read)");
        if (h[5] != 8 || h[6] != 8) return in.fail("sizes of offsets/lengths other than 8");
        const uint64_t p = off + 8 + (ver == 0 ? 16 : 20);  // after flags (v1: + indexed storage K, reserved)
        uint8_t rest[32 + 40];
        if (!in.at(p, rest, sizeof rest)) return false;
        in.base = le(rest, 8);
        sb.root_oh = le(rest + 32 + 8, 8);
        return true;
    }
    return in.fail("no HDF5 signature");
}

// The messages of a version 1 object header, following continuation blocks.
bool read_object_header(In &in, uint64_t addr, std::vector<Message> &out)
{
    uint8_t pre[16];
    if (!in.at(addr, pre, 16)) return false;
    if (std::memcmp(pre, "OHDR", 4) == 0) return in.fail("version 2 object headers are not read");
    if (pre[0] != 1) return in.fail("object header version " + std::to_string(pre[0]));
    const unsigned nmsgs = (unsigned)le(pre + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> chunks = {{addr + 16, le(pre + 8, 4)}};
    for (size_t c = 0; c < chunks.size() && out.size() < nmsgs; c++) {
        if (chunks.size() > 4096) return in.fail("too many continuation blocks");
        std::vector<uint8_t> buf(chunks[c].second);
        if (!buf.empty() && !in.at(chunks[c].first, buf.data(), buf.size())) return false;
        size_t p = 0;
        while (p + 8 <= buf.size() && out.size() < nmsgs) {
            const unsigned type = (unsigned)le(&buf[p], 2);
            const size_t len = (size_t)le(&buf[p + 2], 2);
            if (p + 8 + len > buf.size()) return in.fail("object header message overruns its block");
            Message m{type, std::vector<uint8_t>(buf.begin() + p + 8, buf.begin() + p + 8 + len)};
            if (type == 0x0010) {
                if (len < 16) return in.fail("short continuation message");
                chunks.push_back({le(m.data.data(), 8), le(m.data.data() + 8, 8)});
            }
            out.push_back(std::move(m));
            p += 8 + len;
        }
    }
    return true;
}

const Message *find(const std::vector<Message> &ms, unsigned type)
{
    for (const Message &m : ms)
        if (m.type == type) return &m;
    return nullptr;
}

struct Heap {
    uint64_t data = 0, size = 0;
};

bool read_name(In &in, const Heap &h, uint64_t off, std::string &name)
{
    if (off >= h.size) return in.fail("name offset outside the local heap");
    const size_t n = (size_t)std::min<uint64_t>(h.size - off, 1024);
    std::vector<char> s(n + 1, 0);
    if (!in.at(h.data + off, s.data(), n)) return false;
    name.assign(s.data());
    return true;
}

// Every (name, object header) of a symbol-table group's B-tree.
bool walk_group(In &in, uint64_t node, const Heap &heap, int depth,
                std::vector<std::pair<std::string, uint64_t>> &out)
{
    if (depth > 64) return in.fail("group B-tree too deep");
    uint8_t h[24];
    if (!in.at(node, h, 24)) return false;
    if (std::memcmp(h, "TREE", 4) != 0) return in.fail("bad B-tree node signature");
    if (h[4] != 0) return in.fail("not a group B-tree node");
    const int level = h[5];
    const unsigned used = (unsigned)le(h + 6, 2);
    std::vector<uint8_t> kc((size_t)used * 16 + 8);
    if (!in.at(node + 24, kc.data(), kc.size())) return false;
    for (unsigned i = 0; i < used; i++) {
        const uint64_t child = le(&kc[8 + (size_t)i * 16], 8);
        if (level > 0) {
            if (!walk_group(in, child, heap, depth + 1, out)) return false;
            continue;
        }
        uint8_t sh[8];
        if (!in.at(child, sh, 8)) return false;
        if (std::memcmp(sh, "SNOD", 4) != 0) return in.fail("bad symbol table node signature");
        const unsigned nsym = (unsigned)le(sh + 6, 2);
        std::vector<uint8_t> ents((size_t)nsym * 40);
        if (!ents.empty() && !in.at(child + 8, ents.data(), ents.size())) return false;
        for (unsigned j = 0; j < nsym; j++) {
            std::string name;
            if (!read_name(in, heap, le(&ents[(size_t)j * 40], 8), name)) return false;
            out.push_back({name, le(&ents[(size_t)j * 40 + 8], 8)});
        }
    }
    return true;
}

// A float dataset of the root group, converted to double.  With out ==
// nullptr only the shape is returned.
bool read_dataset(In &in, const char *want, int &rank, uint64_t dims[8], std::vector<double> *out)
{
    Superblock sb;
    if (!read_superblock(in, sb)) return false;
    std::vector<Message> root;
    if (!read_object_header(in, sb.root_oh, root)) return false;
    const Message *st = find(root, 0x0011);
    if (!st || st->data.size() < 16) return in.fail("root group has no symbol table (link-message groups are not read)");
    Heap heap;
    {
        uint8_t h[32];
        if (!in.at(le(st->data.data() + 8, 8), h, 32)) return false;
        if (std::memcmp(h, "HEAP", 4) != 0) return in.fail("bad local heap signature");
        heap.size = le(h + 8, 8);
        heap.data = le(h + 24, 8);
    }
    std::vector<std::pair<std::string, uint64_t>> ents;
    if (!walk_group(in, le(st->data.data(), 8), heap, 0, ents)) return false;
    uint64_t oh = kUndef;
    for (auto &e : ents)
        if (e.first == want) oh = e.second;
    if (oh == kUndef) return in.fail(std::string("no dataset \"") + want + "\" in the root group");
    std::vector<Message> ms;
    if (!read_object_header(in, oh, ms)) return false;
    const Message *sp = find(ms, 0x0001), *ty = find(ms, 0x0003), *ly = find(ms, 0x0008);
    if (!sp || !ty || !ly) return in.fail(std::string("\"") + want + "\" is not a dataset");
    if (find(ms, 0x000B)) return in.fail("filtered (compressed) datasets are not read");
    if (find(ms, 0x0007)) return in.fail("external storage is not read");
    // dataspace
    const std::vector<uint8_t> &s = sp->data;
    if (s.size() < 4) return in.fail("short dataspace message");
    rank = s[1];
    if (rank > 8) return in.fail("rank above 8");
    const size_t d0 = s[0] == 1 ? 8 : s[0] == 2 ? 4 : 0;
    if (!d0) return in.fail("dataspace version " + std::to_string(s[0]));
    if (s.size() < d0 + (size_t)rank * 8) return in.fail("short dataspace message");
    uint64_t count = 1;
    for (int i = 0; i < rank; i++) {
        dims[i] = le(&s[d0 + (size_t)i * 8], 8);
        count *= dims[i];
    }
    // datatype: IEEE float32/float64
    const std::vector<uint8_t> &t = ty->data;
    if (t.size() < 20 || (t[0] & 0x0f) != 1) return in.fail("datatype is not floating point");
    const bool be = (t[1] & 1) != 0;
    const uint32_t esize = (uint32_t)le(&t[4], 4);
    const unsigned prec = (unsigned)le(&t[10], 2), ebits = t[13], mbits = t[15];
    const bool f64 = esize == 8 && prec == 64 && ebits == 11 && mbits == 52;
    const bool f32 = esize == 4 && prec == 32 && ebits == 8 && mbits == 23;
    if (!f64 && !f32) return in.fail("floating-point type other than IEEE float32/float64");
    // every stored form keeps its values inside the file: a larger dataspace
    // is a damaged file, not an allocation to attempt
    {
        uint64_t c = 1;
        for (int i = 0; i < rank; i++) {
            if (dims[i] && c > in.size / dims[i]) return in.fail("dataspace larger than the file");
            c *= dims[i];
        }
        if (c > in.size / esize) return in.fail("dataspace larger than the file");
    }
    if (!out) return true;
    // layout
    const std::vector<uint8_t> &l = ly->data;
    if (l.size() < 2) return in.fail("short layout message");
    const uint64_t need = count * esize;
    std::vector<uint8_t> raw;
    if (l[0] == 1 || l[0] == 2) {
        if (l.size() < 8) return in.fail("short layout message");
        const int nd = l[1], cls = l[2];
        if (cls == 1) {
            if (l.size() < 16) return in.fail("short layout message");
            const uint64_t addr = le(&l[8], 8);
            raw.resize(need);
            if (need && !in.at(addr, raw.data(), need)) return false;
        } else if (cls == 0) {
            const size_t p = 8 + (size_t)nd * 4;
            if (l.size() < p + 4) return in.fail("short layout message");
            const uint64_t n = le(&l[p], 4);
            if (n < need || l.size() < p + 4 + need) return in.fail("compact data shorter than the dataspace");
            raw.assign(l.begin() + p + 4, l.begin() + p + 4 + need);
        } else {
            return in.fail("chunked datasets are not read");
        }
    } else if (l[0] == 3) {
        if (l[1] == 1) {
            if (l.size() < 18) return in.fail("short layout message");
            const uint64_t addr = le(&l[2], 8), n = le(&l[10], 8);
            if (n < need) return in.fail("contiguous storage shorter than the dataspace");
            if (f64 && !be && host_is_le()) {  // the common case: the bytes are the doubles
                out->resize(count);
                return !need || in.at(addr, out->data(), need);
            }
            raw.resize(need);
            if (need && !in.at(addr, raw.data(), need)) return false;
        } else if (l[1] == 0) {
            if (l.size() < 4) return in.fail("short layout message");
            const uint64_t n = le(&l[2], 2);
            if (n < need || l.size() < 4 + need) return in.fail("compact data shorter than the dataspace");
            raw.assign(l.begin() + 4, l.begin() + 4 + need);
        } else {
            return in.fail("chunked or virtual datasets are not read");
        }
    } else {
        return in.fail("layout message version " + std::to_string(l[0]));
    }
    out->resize(count);
    for (uint64_t i = 0; i < count; i++) {
        const uint8_t *p = &raw[i * esize];
        uint64_t bits = 0;
        for (uint32_t k = 0; k < esize; k++) bits |= (uint64_t)p[be ? esize - 1 - k : k] << (8 * k);
        if (f64) {
            std::memcpy(&(*out)[i], &bits, 8);
        } else {
            const uint32_t b32 = (uint32_t)bits;
            float f;
            std::memcpy(&f, &b32, 4);
            (*out)[i] = f;
        }
    }
    return true;
}

bool field_dims(int ndim, const int64_t *n, uint64_t dims[3], std::string &err)
{
    if ((ndim != 2 && ndim != 3) || !n) {
        err = "h5: ndim must be 2 or 3";
        return false;
    }
    for (int i = 0; i < ndim; i++) {
        if (n[i] < 1) {
            err = "h5: sizes must be positive";
            return false;
        }
        dims[ndim - 1 - i] = (uint64_t)n[i];  // Julia's (nx, ny[, nz]) as the HDF5 (.., ny, nx)
    }
    return true;
}

int write_field(const char *path, int ndim, const int64_t *n, const double *psi, std::string &err)
{
    if (!path || !psi) {
        err = "h5: null path or field";
        return GPSS_EINVAL;
    }
    uint64_t dims[3];
    if (!field_dims(ndim, n, dims, err)) return GPSS_EINVAL;
    uint64_t count = 1;
    for (int i = 0; i < ndim; i++) count *= dims[i];
    std::vector<double> re(count), im(count);
    for (uint64_t i = 0; i < count; i++) {
        re[i] = psi[2 * i];
        im[i] = psi[2 * i + 1];
    }
    return write_file(path, ndim, dims, {{"re", re.data()}, {"im", im.data()}}, err);
}

int read_field(const char *path, int ndim, const int64_t *n, double *psi, std::string &err)
{
    if (!path || !psi) {
        err = "h5: null path or field";
        return GPSS_EINVAL;
    }
    uint64_t want[3];
    if (!field_dims(ndim, n, want, err)) return GPSS_EINVAL;
    std::vector<double> part[2];
    const char *names[2] = {"re", "im"};
    for (int k = 0; k < 2; k++) {
        In in;
        int rank = 0;
        uint64_t dims[8];
        if (!in.open(path) || !read_dataset(in, names[k], rank, dims, &part[k])) {
            err = in.err;
            return GPSS_EIO;
        }
        bool same = rank == ndim;
        for (int i = 0; same && i < ndim; i++) same = dims[i] == want[i];
        if (!same) {
            err = std::string("h5: dataset \"") + names[k] + "\" does not have the field's shape";
            return GPSS_EINVAL;
        }
    }
    for (size_t i = 0; i < part[0].size(); i++) {
        psi[2 * i] = part[0][i];
        psi[2 * i + 1] = part[1][i];
    }
    return GPSS_OK;
}

// calls without a context leave their message for gpss_last_error(NULL)
int ctxless(int rc, const std::string &err)
{
    return rc == GPSS_OK ? rc : gpss::fail(nullptr, rc, "%s", err.c_str());
}

int read_dataset_entry(const char *path, const char *name, int *rank, int64_t *dims, double *out, int64_t cap)
{
    In in;
    int r = 0;
    uint64_t d[8];
    std::vector<double> v;
    if (!in.open(path) || !read_dataset(in, name, r, d, out ? &v : nullptr)) return ctxless(GPSS_EIO, in.err);
    *rank = r;
    for (int i = 0; i < r; i++) dims[i] = (int64_t)d[i];
    if (out) {
        if ((int64_t)v.size() > cap) return ctxless(GPSS_EINVAL, "h5: output buffer too small");
        std::memcpy(out, v.data(), v.size() * sizeof(double));
    }
    return GPSS_OK;
}

int write_ctx(gpss_ctx *c, const char *path)
{
    std::vector<double> psi((size_t)c->total * 2);
    const int rc = gpss_download(c, psi.data());
    if (rc != GPSS_OK) return rc;
    std::string err;
    const int w = write_field(path, c->ndim, c->n, psi.data(), err);
    return w == GPSS_OK ? w : gpss::fail(c, w, "%s", err.c_str());
}

int read_ctx(gpss_ctx *c, const char *path)
{
    std::vector<double> psi((size_t)c->total * 2);
    std::string err;
    const int r = read_field(path, c->ndim, c->n, psi.data(), err);
    if (r != GPSS_OK) return gpss::fail(c, r, "%s", err.c_str());
    return gpss_upload(c, psi.data());
}

// No C++ exception leaves an entry point: a failed host allocation is ENOMEM.
template <typename F> int guarded(gpss_ctx *c, F body)
{
    try {
        return body();
    } catch (const std::bad_alloc &) {
        return gpss::fail(c, GPSS_ENOMEM, "h5: host allocation failed");
    } catch (...) {
        return gpss::fail(c, GPSS_EIO, "h5: unexpected failure");
    }
}

}  // namespace

extern "C" {

int gpss_h5_write_field(const char *path, int ndim, const int64_t *n, const double *psi)
{
    return guarded(nullptr, [&] {
        std::string err;
        return ctxless(write_field(path, ndim, n, psi, err), err);
    });
}

int gpss_h5_read_field(const char *path, int ndim, const int64_t *n, double *psi)
{
    return guarded(nullptr, [&] {
        std::string err;
        return ctxless(read_field(path, ndim, n, psi, err), err);
    });
}

int gpss_h5_read_dataset(const char *path, const char *name, int *rank, int64_t *dims, double *out, int64_t cap)
{
    if (!path || !name || !rank || !dims) return ctxless(GPSS_EINVAL, "h5: null argument");
    return guarded(nullptr, [&] { return read_dataset_entry(path, name, rank, dims, out, cap); });
}

int gpss_write_h5(gpss_ctx *c, const char *path)
{
    if (!c) return GPSS_EINVAL;
    return guarded(c, [&] { return write_ctx(c, path); });
}

int gpss_read_h5(gpss_ctx *c, const char *path)
{
    if (!c) return GPSS_EINVAL;
    return guarded(c, [&] { return read_ctx(c, path); });
}

}  // extern "C"
