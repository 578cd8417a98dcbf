// HDF5 file I/O of the reference's file path (include/io.h:35-197, dispatch by element
// type include/hpdbscan.h:300-356), written for this project from the published HDF5
// file format specification because libhdf5 is not available to this build.  It covers
// what that path needs:
//
//   read   a 2-D dataset of one of the ten element types: superblock versions 0-3,
//          object headers version 1 and 2 (with continuation blocks), groups held as a
//          symbol table (v1 B-tree + local heap) or as compact link messages,
//          fixed-point and IEEE floating-point data of either byte order, compact,
//          contiguous and chunked layouts (v1 B-tree chunk index, no filters), fill
//          values for storage never written;
//   write  the labels as a 1-D int64 dataset (the reference's H5T_NATIVE_LONG): into a
//          new file, into an existing dataset of that name (the first n elements, with
//          the reference's integer / floating-point conversion), or as a new dataset of
//          a symbol-table group (the layout libhdf5 and h5py write by default).
//
// Status and messages follow the reference: "Could not open <path>", "Could not open
// dataset <name>", "Data in dataset <name> should be a matrix", the "Unsupported ..."
// element types (std::invalid_argument there), "Failed to read data" and "Failed to
// write data, target data set is probably of wrong size or type" (std::runtime_error).
// A file feature outside this subset is reported with the reference message of the
// step that meets it and the feature in parentheses.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hpdbscan_gb300.h"

namespace hpd {
void set_last_error(const std::string& msg);  // hpd_capi.cu: the message of hpd_last_error()
}

namespace {

constexpr uint64_t kUndef = ~0ull;
const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// A structure this subset does not read, or a broken file.
struct Bad : std::runtime_error {
    using std::runtime_error::runtime_error;
};

uint64_t rd(const unsigned char* p, int bytes) {
    uint64_t v = 0;
    for (int i = bytes - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

void wr(unsigned char* p, uint64_t v, int bytes) {
    for (int i = 0; i < bytes; ++i) p[i] = (unsigned char)(v >> (8 * i));
}

void need(uint64_t have, uint64_t want) {
    if (have < want) throw Bad("truncated header message");
}

// The file mapped copy-on-write, plus the bytes appended by a write.  Addresses are
// relative to the superblock's base address, as in the format.
struct File {
    int fd = -1;
    unsigned char* map = nullptr;
    uint64_t size = 0;               // bytes of the file as opened
    std::vector<unsigned char> tail; // appended at `size`
    std::vector<std::pair<uint64_t, uint64_t>> dirty;  // modified [lo, hi) below `size`
    int so = 8, sl = 8;              // size of offsets, size of lengths
    uint64_t sb = 0, base = 0, eoa = 0;  // eoa: from the start of the file
    int sb_version = 0, leaf_k = 4, internal_k = 16;
    uint64_t root_header = kUndef, root_btree = kUndef, root_heap = kUndef;

    File() = default;
    File(const File&) = delete;
    File& operator=(const File&) = delete;
    ~File() {
        if (map) munmap(map, size);
        if (fd >= 0) close(fd);
    }
    uint64_t end() const { return size + tail.size(); }
    unsigned char* ptr(uint64_t addr, uint64_t len) {
        if (addr == kUndef) throw Bad("undefined address");
        const uint64_t a = addr + base;
        if (a < addr) throw Bad("address out of the file");
        if (a < size) {
            if (len > size - a) throw Bad("address out of the file");
            return map + a;
        }
        if (a - size > tail.size() || len > tail.size() - (a - size)) throw Bad("address out of the file");
        return tail.data() + (a - size);
    }
    const unsigned char* at(uint64_t addr, uint64_t len) const { return const_cast<File*>(this)->ptr(addr, len); }
    unsigned char* mut(uint64_t addr, uint64_t len) {  // bytes that will be written back
        unsigned char* p = ptr(addr, len);
        if (addr + base < size) dirty.push_back({addr + base, addr + base + len});
        return p;
    }
    uint64_t alloc(uint64_t bytes) {  // zeroed block at the end of the file, 8-byte aligned
        uint64_t a = std::max(end(), eoa);
        a = (a + 7) & ~7ull;
        tail.resize(a - size + bytes, 0);
        return a - base;
    }
    uint64_t off(const unsigned char*& p) const {
        const uint64_t v = rd(p, so);
        p += so;
        return v;
    }
    uint64_t len(const unsigned char*& p) const {
        const uint64_t v = rd(p, sl);
        p += sl;
        return v;
    }
};

// Maps the file and reads its superblock; false when it is not an HDF5 file.
bool open_file(const std::string& path, File& f, bool writable) {
    f.fd = open(path.c_str(), O_RDONLY);
    if (f.fd < 0) return false;
    struct stat st;
    if (fstat(f.fd, &st) != 0 || !S_ISREG(st.st_mode) || st.st_size < 8) return false;
    f.size = (uint64_t)st.st_size;
    void* m = mmap(nullptr, f.size, PROT_READ | (writable ? PROT_WRITE : 0), MAP_PRIVATE, f.fd, 0);
    if (m == MAP_FAILED) {
        f.size = 0;
        return false;
    }
    f.map = static_cast<unsigned char*>(m);
    f.sb = kUndef;  // at 0, or at 512 bytes times a power of two (after a user block)
    for (uint64_t a = 0; a + 8 <= f.size; a = a ? a * 2 : 512)
        if (std::memcmp(f.map + a, kSig, 8) == 0) {
            f.sb = a;
            break;
        }
    if (f.sb == kUndef || f.size - f.sb < 48) return false;
    const unsigned char* p = f.map + f.sb + 8;
    f.sb_version = p[0];
    if (f.sb_version == 0 || f.sb_version == 1) {
        if (f.size - f.sb < 100) return false;
        f.so = p[5];
        f.sl = p[6];
        if (f.so != 8 || f.sl != 8) throw Bad("offsets or lengths other than 8 bytes");
        f.leaf_k = (int)rd(p + 8, 2);
        f.internal_k = (int)rd(p + 10, 2);
        p += 16 + (f.sb_version == 1 ? 4 : 0);
        f.base = f.off(p);
        f.off(p);  // free-space information
        f.eoa = f.off(p);
        f.off(p);  // driver information
        f.off(p);  // root entry: link name offset
        f.root_header = f.off(p);
        const uint32_t cache = (uint32_t)rd(p, 4);
        p += 8;
        if (cache == 1) {
            f.root_btree = f.off(p);
            f.root_heap = f.off(p);
        }
    } else if (f.sb_version == 2 || f.sb_version == 3) {
        f.so = p[1];
        f.sl = p[2];
        if (f.so != 8 || f.sl != 8) throw Bad("offsets or lengths other than 8 bytes");
        p += 4;
        f.base = f.off(p);
        f.off(p);  // superblock extension
        f.eoa = f.off(p);
        f.root_header = f.off(p);
    } else {
        throw Bad("superblock version " + std::to_string(f.sb_version));
    }
    // the stored end-of-file address counts from the start of the file (user block
    // included), unlike every other address, which is relative to the base address
    if (f.eoa != kUndef && f.eoa > f.size) throw Bad("truncated file");
    return true;
}

struct Msg {
    int type;
    int flags;
    uint64_t addr;  // of the message data
    uint64_t size;
};

// Header messages of the object at `addr`, continuation blocks followed; both header versions.
std::vector<Msg> messages(const File& f, uint64_t addr) {
    std::vector<Msg> out;
    std::vector<std::pair<uint64_t, uint64_t>> blocks;  // (address, length) of message blocks
    const unsigned char* h = f.at(addr, 16);
    if (std::memcmp(h, "OHDR", 4) == 0) {
        if (h[4] != 2) throw Bad("object header version " + std::to_string(h[4]));
        const int flags = h[5];
        const uint64_t pos = 6 + ((flags & 0x20) ? 16 : 0) + ((flags & 0x10) ? 4 : 0);
        const int sz = 1 << (flags & 3);
        blocks.push_back({addr + pos + sz, rd(f.at(addr + pos, sz), sz)});
        const uint64_t head = 4 + ((flags & 4) ? 2 : 0);
        for (size_t b = 0; b < blocks.size(); ++b) {
            if (b > 64) throw Bad("too many object header continuations");
            uint64_t a = blocks[b].first;
            const uint64_t end = a + blocks[b].second;
            while (a + head <= end) {
                const unsigned char* m = f.at(a, head);
                const Msg msg{m[0], m[3], a + head, rd(m + 1, 2)};
                if (msg.addr + msg.size > end) break;
                if (msg.type == 0x10) {  // continuation: "OCHK", messages, checksum
                    need(msg.size, 16);
                    const unsigned char* c = f.at(msg.addr, 16);
                    const uint64_t ca = f.off(c), cl = f.len(c);
                    if (cl < 8 || std::memcmp(f.at(ca, 4), "OCHK", 4) != 0) throw Bad("bad continuation block");
                    blocks.push_back({ca + 4, cl - 8});
                } else {
                    out.push_back(msg);
                }
                a = msg.addr + msg.size;
            }
        }
        return out;
    }
    if (h[0] != 1) throw Bad("object header version " + std::to_string(h[0]));
    const uint64_t nmsg = rd(h + 2, 2);
    blocks.push_back({addr + 16, rd(h + 8, 4)});
    uint64_t seen = 0;
    for (size_t b = 0; b < blocks.size() && seen < nmsg; ++b) {
        if (b > 64) throw Bad("too many object header continuations");
        uint64_t a = blocks[b].first;
        const uint64_t end = a + blocks[b].second;
        while (a + 8 <= end && seen < nmsg) {
            const unsigned char* m = f.at(a, 8);
            const Msg msg{(int)rd(m, 2), m[4], a + 8, rd(m + 2, 2)};
            f.at(msg.addr, msg.size);
            ++seen;
            if (msg.type == 0x10) {
                need(msg.size, 16);
                const unsigned char* c = f.at(msg.addr, 16);
                const uint64_t ca = f.off(c), cl = f.len(c);
                blocks.push_back({ca, cl});
            } else {
                out.push_back(msg);
            }
            a = msg.addr + ((msg.size + 7) & ~7ull);
        }
    }
    return out;
}

// ------------------------------------------------------------------ groups

struct Heap {
    uint64_t header, data, size;
};

Heap local_heap(const File& f, uint64_t addr) {
    const unsigned char* h = f.at(addr, 32);
    if (std::memcmp(h, "HEAP", 4) != 0) throw Bad("bad local heap");
    const unsigned char* p = h + 8;
    Heap hp{addr, 0, 0};
    hp.size = f.len(p);
    f.len(p);  // free list
    hp.data = f.off(p);
    f.at(hp.data, hp.size);
    return hp;
}

std::string heap_name(const File& f, const Heap& hp, uint64_t off) {
    if (off >= hp.size) throw Bad("name outside the local heap");
    const unsigned char* s = f.at(hp.data, hp.size);
    const void* z = std::memchr(s + off, 0, hp.size - off);
    if (!z) throw Bad("unterminated name in the local heap");
    return std::string(reinterpret_cast<const char*>(s + off), static_cast<const unsigned char*>(z) - (s + off));
}

constexpr uint64_t kSnodEntry = 40;

struct SymTab {
    uint64_t btree = kUndef, heap = kUndef;
};

// Object header address of `name` in a symbol-table group (group B-tree of SNODs).
uint64_t find_in_btree(const File& f, uint64_t node, const Heap& hp, const std::string& name, int depth = 0) {
    if (depth > 32) throw Bad("group B-tree too deep");
    const unsigned char* t = f.at(node, 24);
    if (std::memcmp(t, "TREE", 4) != 0 || t[4] != 0) throw Bad("bad group B-tree node");
    const int level = t[5];
    const uint64_t used = rd(t + 6, 2);
    const unsigned char* kc = f.at(node + 24, (2 * used + 1) * 8);  // key0 child0 key1 ... key_used
    for (uint64_t i = 0; i < used; ++i) {
        if (name.compare(heap_name(f, hp, rd(kc + 16 * i + 16, 8))) > 0) continue;
        const uint64_t child = rd(kc + 16 * i + 8, 8);
        if (level > 0) return find_in_btree(f, child, hp, name, depth + 1);
        const unsigned char* s = f.at(child, 8);
        if (std::memcmp(s, "SNOD", 4) != 0) throw Bad("bad symbol table node");
        const uint64_t n = rd(s + 6, 2);
        const unsigned char* e = f.at(child + 8, n * kSnodEntry);
        for (uint64_t k = 0; k < n; ++k, e += kSnodEntry)
            if (name == heap_name(f, hp, rd(e, 8))) return rd(e + 8, 8);
        return kUndef;
    }
    return kUndef;
}

// The symbol table of a group object; undefined for a group held as link messages.
SymTab symbol_table(const File& f, uint64_t obj) {
    SymTab st;
    if (obj == f.root_header && f.root_btree != kUndef) return {f.root_btree, f.root_heap};
    for (const Msg& m : messages(f, obj))
        if (m.type == 0x11) {
            need(m.size, 16);
            const unsigned char* p = f.at(m.addr, 16);
            st.btree = f.off(p);
            st.heap = f.off(p);
        }
    return st;
}

// Hard link `name` among the link messages of a group object (compact link storage).
uint64_t find_link(const File& f, uint64_t obj, const std::string& name) {
    uint64_t found = kUndef;
    for (const Msg& m : messages(f, obj)) {
        const unsigned char* p = f.at(m.addr, m.size);
        const unsigned char* e = p + m.size;
        if (m.type == 0x02) {  // link info: dense storage when the fractal heap address is defined
            need(m.size, 2);
            const unsigned char* q = p + 2 + ((p[1] & 1) ? 8 : 0);
            need(e - q, 8);
            if (rd(q, 8) != kUndef) throw Bad("groups with dense link storage");
        }
        if (m.type != 0x06) continue;
        need(m.size, 3);
        const int flags = p[1];
        p += 2;
        int ltype = 0;
        if (flags & 0x08) ltype = *p++;
        if (flags & 0x04) p += 8;
        if (flags & 0x10) ++p;
        const int lb = 1 << (flags & 3);
        need(e - p, lb);
        const uint64_t ln = rd(p, lb);
        p += lb;
        need(e - p, ln);
        const std::string lname(reinterpret_cast<const char*>(p), ln);
        p += ln;
        if (ltype == 0 && lname == name) {
            need(e - p, 8);
            found = rd(p, 8);
        }
    }
    return found;
}

std::vector<std::string> split_path(const std::string& path) {
    std::vector<std::string> parts;
    size_t pos = 0;
    while (pos <= path.size()) {
        size_t next = path.find('/', pos);
        if (next == std::string::npos) next = path.size();
        const std::string part = path.substr(pos, next - pos);
        if (!part.empty() && part != ".") parts.push_back(part);
        pos = next + 1;
    }
    return parts;
}

// Object header address of the child `name` of group `obj` (kUndef when absent).
uint64_t child_of(const File& f, uint64_t obj, const std::string& name) {
    const SymTab st = symbol_table(f, obj);
    if (st.btree != kUndef) return find_in_btree(f, st.btree, local_heap(f, st.heap), name);
    return find_link(f, obj, name);
}

uint64_t find_object(const File& f, const std::vector<std::string>& parts) {
    uint64_t obj = f.root_header;
    for (const std::string& part : parts) {
        obj = child_of(f, obj, part);
        if (obj == kUndef) return kUndef;
    }
    return obj;
}

// ------------------------------------------------------------------ datasets

struct Dtype {
    int cls = -1;        // 0 fixed-point, 1 floating-point, other classes unsupported
    uint32_t size = 0;   // bytes per element
    bool big = false;    // big-endian
    bool sign = false;   // fixed-point: two's complement
    int offset = 0, precision = 0;
    bool ieee = false;   // floating-point: the IEEE 754 binary32 / binary64 layout
};

struct Dataset {
    uint64_t header = kUndef;
    int rank = -1;
    std::vector<uint64_t> dims;
    Dtype type;
    bool has_type = false, has_layout = false, filtered = false, external = false;
    int layout_class = -1;            // 0 compact, 1 contiguous, 2 chunked
    uint64_t layout_msg = kUndef;     // address of the layout message's data
    int layout_version = 0;
    uint64_t data = kUndef, data_size = 0;  // compact: bytes in the message; contiguous: in the file
    std::vector<uint64_t> chunk;      // chunk extent per dimension
    uint64_t chunk_index = kUndef;    // v1 B-tree of chunks
    std::vector<unsigned char> fill;  // fill value bytes (empty: zeros)
};

Dtype parse_type(const File& f, const Msg& m) {
    need(m.size, 8);
    const unsigned char* p = f.at(m.addr, m.size);
    Dtype t;
    t.cls = p[0] & 15;
    t.size = (uint32_t)rd(p + 4, 4);
    if (t.cls == 0) {
        need(m.size, 12);
        t.big = p[1] & 1;
        t.sign = p[1] & 8;
        t.offset = (int)rd(p + 8, 2);
        t.precision = (int)rd(p + 10, 2);
    } else if (t.cls == 1) {
        need(m.size, 20);
        t.big = p[1] & 1;
        const bool vax = p[1] & 0x40;
        const int norm = (p[1] >> 4) & 3, sign_loc = p[2];
        t.offset = (int)rd(p + 8, 2);
        t.precision = (int)rd(p + 10, 2);
        const int exp_loc = p[12], exp_size = p[13], mant_loc = p[14], mant_size = p[15];
        const uint32_t bias = (uint32_t)rd(p + 16, 4);
        t.ieee = !vax && norm == 2 && t.offset == 0 && mant_loc == 0 &&
                 ((t.precision == 32 && t.size == 4 && sign_loc == 31 && exp_loc == 23 && exp_size == 8 &&
                   mant_size == 23 && bias == 127) ||
                  (t.precision == 64 && t.size == 8 && sign_loc == 63 && exp_loc == 52 && exp_size == 11 &&
                   mant_size == 52 && bias == 1023));
    }
    return t;
}

Dataset parse_dataset(const File& f, uint64_t header) {
    Dataset ds;
    ds.header = header;
    std::vector<unsigned char> old_fill;
    bool new_fill_seen = false;
    for (const Msg& m : messages(f, header)) {
        const unsigned char* p = f.at(m.addr, m.size);
        if ((m.type == 0x01 || m.type == 0x03) && (m.flags & 2)) throw Bad("shared dataspace or datatype messages");
        if (m.type == 0x01) {  // dataspace
            need(m.size, 8);
            const int version = p[0];
            ds.rank = p[1];
            uint64_t pos;
            if (version == 1) {
                pos = 8;
            } else if (version == 2) {
                pos = 4;
                if (p[3] == 2) ds.rank = 0;  // null dataspace
            } else {
                throw Bad("dataspace version " + std::to_string(version));
            }
            need(m.size, pos + 8 * (uint64_t)ds.rank);
            for (int i = 0; i < ds.rank; ++i) ds.dims.push_back(rd(p + pos + 8 * i, 8));
        } else if (m.type == 0x03) {
            ds.type = parse_type(f, m);
            ds.has_type = true;
        } else if (m.type == 0x04) {  // fill value (old): size, value
            need(m.size, 4);
            const uint64_t n = rd(p, 4);
            need(m.size, 4 + n);
            old_fill.assign(p + 4, p + 4 + n);
        } else if (m.type == 0x05) {  // fill value
            need(m.size, 2);
            new_fill_seen = true;
            const int version = p[0];
            uint64_t pos = 0;
            bool defined = false;
            if (version == 1 || version == 2) {
                need(m.size, 4);
                defined = p[3] != 0;
                pos = 4;
                if (version == 1 || defined) {
                    need(m.size, 8);
                    const uint64_t n = rd(p + 4, 4);
                    need(m.size, 8 + n);
                    if (defined) ds.fill.assign(p + 8, p + 8 + n);
                }
            } else if (version == 3) {
                defined = p[1] & 0x20;
                pos = 2;
                if (defined) {
                    need(m.size, 6);
                    const uint64_t n = rd(p + 2, 4);
                    need(m.size, 6 + n);
                    ds.fill.assign(p + 6, p + 6 + n);
                }
            }
            (void)pos;
        } else if (m.type == 0x07) {
            ds.external = true;
        } else if (m.type == 0x08) {  // data layout
            need(m.size, 2);
            ds.has_layout = true;
            ds.layout_msg = m.addr;
            ds.layout_version = p[0];
            if (ds.layout_version == 3) {
                ds.layout_class = p[1];
                if (ds.layout_class == 0) {
                    need(m.size, 4);
                    ds.data_size = rd(p + 2, 2);
                    need(m.size, 4 + ds.data_size);
                    ds.data = m.addr + 4;
                } else if (ds.layout_class == 1) {
                    need(m.size, 18);
                    ds.data = rd(p + 2, 8);
                    ds.data_size = rd(p + 10, 8);
                } else if (ds.layout_class == 2) {
                    need(m.size, 3);
                    const int nd = p[2];
                    need(m.size, 11 + 4 * (uint64_t)nd);
                    ds.chunk_index = rd(p + 3, 8);
                    for (int i = 0; i < nd; ++i) ds.chunk.push_back(rd(p + 11 + 4 * i, 4));
                }
            } else if (ds.layout_version == 1 || ds.layout_version == 2) {
                need(m.size, 8);
                const int nd = p[1];
                ds.layout_class = p[2];
                uint64_t pos = 8;
                if (ds.layout_class != 0) {
                    need(m.size, pos + 8);
                    ds.data = ds.layout_class == 1 ? rd(p + pos, 8) : kUndef;
                    if (ds.layout_class == 2) ds.chunk_index = rd(p + pos, 8);
                    pos += 8;
                }
                need(m.size, pos + 4 * (uint64_t)nd);
                for (int i = 0; i < nd; ++i) ds.chunk.push_back(rd(p + pos + 4 * i, 4));
                pos += 4 * (uint64_t)nd;
                if (ds.layout_class == 0) {
                    need(m.size, pos + 4);
                    ds.data_size = rd(p + pos, 4);
                    need(m.size, pos + 4 + ds.data_size);
                    ds.data = m.addr + pos + 4;
                } else if (ds.layout_class == 1) {
                    uint64_t bytes = 1;
                    for (uint64_t c : ds.chunk) bytes *= c;
                    ds.data_size = bytes;
                }
                ds.chunk.clear();
                if (ds.layout_class == 2) {
                    for (int i = 0; i < nd; ++i) ds.chunk.push_back(rd(p + 8 + 8 + 4 * i, 4));
                }
            } else {
                ds.layout_class = -2;  // chunk indexes of the 1.10+ format
            }
        } else if (m.type == 0x0B) {  // filter pipeline
            need(m.size, 2);
            if (p[1] > 0) ds.filtered = true;
        }
    }
    if (!new_fill_seen && !old_fill.empty()) ds.fill = old_fill;
    if (ds.layout_class == 2 && ds.chunk.size() == (size_t)ds.rank + 1) ds.chunk.pop_back();  // element size
    return ds;
}

bool is_dataset(const Dataset& ds) { return ds.has_layout && ds.has_type && ds.rank >= 0; }

bool mul_ok(uint64_t a, uint64_t b, uint64_t& out) {
    if (a && b > std::numeric_limits<uint64_t>::max() / a) return false;
    out = a * b;
    return true;
}

// Every element of the dataset, row-major, in file byte order; storage never written
// reads as the fill value.
void read_elements(const File& f, const Dataset& ds, unsigned char* out, uint64_t count) {
    const uint64_t es = ds.type.size;
    const uint64_t bytes = count * es;
    if (ds.filtered) throw Bad("filtered or compressed datasets");
    if (ds.external) throw Bad("external data files");
    const bool fill = !ds.fill.empty() && ds.fill.size() == es;
    auto fill_all = [&](unsigned char* dst, uint64_t n) {
        if (!fill) {
            std::memset(dst, 0, n * es);
            return;
        }
        for (uint64_t i = 0; i < n; ++i) std::memcpy(dst + i * es, ds.fill.data(), es);
    };
    if (ds.layout_class == 0 || ds.layout_class == 1) {
        if (ds.layout_class == 1 && ds.data == kUndef) {
            fill_all(out, count);
            return;
        }
        if (ds.data_size < bytes) throw Bad("dataset storage smaller than its extent");
        if (bytes) std::memcpy(out, f.at(ds.data, bytes), bytes);
        return;
    }
    if (ds.layout_class != 2) throw Bad("the chunk indexes of the HDF5 1.10 file format");
    if ((int)ds.chunk.size() != ds.rank) throw Bad("bad chunk dimensions");
    fill_all(out, count);
    if (ds.chunk_index == kUndef || count == 0) return;
    uint64_t chunk_elems = 1;
    for (uint64_t c : ds.chunk) {
        if (c == 0 || !mul_ok(chunk_elems, c, chunk_elems)) throw Bad("bad chunk dimensions");
    }
    // depth-first over the chunk B-tree; a chunk's part inside the extent is copied row by row
    std::vector<std::pair<uint64_t, int>> stack = {{ds.chunk_index, 0}};
    const int rank = ds.rank;
    const uint64_t key_size = 8 + 8 * (uint64_t)(rank + 1);
    uint64_t visited = 0;
    while (!stack.empty()) {
        const auto [node, depth] = stack.back();
        stack.pop_back();
        if (depth > 32 || ++visited > (1u << 26)) throw Bad("bad chunk B-tree");
        const unsigned char* t = f.at(node, 24);
        if (std::memcmp(t, "TREE", 4) != 0 || t[4] != 1) throw Bad("bad chunk B-tree node");
        const int level = t[5];
        const uint64_t used = rd(t + 6, 2);
        const unsigned char* p = f.at(node + 24, used * (key_size + 8) + key_size);
        for (uint64_t i = 0; i < used; ++i) {
            const unsigned char* key = p + i * (key_size + 8);
            const uint64_t child = rd(key + key_size, 8);
            if (level > 0) {
                stack.push_back({child, depth + 1});
                continue;
            }
            if (rd(key + 4, 4) != 0) throw Bad("filtered or compressed datasets");
            if (rd(key, 4) < chunk_elems * es) throw Bad("short chunk");
            const unsigned char* src = f.at(child, chunk_elems * es);
            std::vector<uint64_t> origin(rank);
            for (int k = 0; k < rank; ++k) {
                origin[k] = rd(key + 8 + 8 * k, 8);
                if (origin[k] >= ds.dims[k]) throw Bad("chunk outside the dataset");
            }
            const uint64_t row = std::min(ds.chunk[rank - 1], ds.dims[rank - 1] - origin[rank - 1]);
            std::vector<uint64_t> idx(rank, 0);  // chunk-local index of the row start (last dim 0)
            while (true) {
                bool inside = true;
                uint64_t lin = 0, loc = 0;
                for (int k = 0; k < rank; ++k) {
                    const uint64_t g = origin[k] + idx[k];
                    if (g >= ds.dims[k]) inside = false;
                    lin = lin * ds.dims[k] + g;
                    loc = loc * ds.chunk[k] + idx[k];
                }
                if (inside) std::memcpy(out + lin * es, src + loc * es, row * es);
                int k = rank - 2;
                for (; k >= 0; --k) {
                    if (++idx[k] < ds.chunk[k]) break;
                    idx[k] = 0;
                }
                if (k < 0) break;
            }
        }
    }
}

void swap_bytes(unsigned char* p, uint64_t count, uint32_t es) {
    for (uint64_t i = 0; i < count; ++i, p += es) std::reverse(p, p + es);
}

int fail(int code, const std::string& msg) {
    hpd::set_last_error(msg);
    return code;
}

std::string why(const char* base, const std::exception& e) { return std::string(base) + " (" + e.what() + ")"; }

// The reference's element-type dispatch (include/hpdbscan.h:309-355).
int dtype_of(const Dtype& t, int32_t* dtype) {
    if (t.cls == 0) {
        static const int s[] = {HPD_I8, HPD_I16, HPD_I32, HPD_I64}, u[] = {HPD_U8, HPD_U16, HPD_U32, HPD_U64};
        const int k = t.precision == 8 ? 0 : t.precision == 16 ? 1 : t.precision == 32 ? 2 : t.precision == 64 ? 3 : -1;
        if (k < 0)
            return fail(HPD_ERR_UNSUPPORTED, t.sign ? "Unsupported signed integer precision"
                                                    : "Unsupported unsigned integer precision");
        *dtype = t.sign ? s[k] : u[k];
        return HPD_OK;
    }
    if (t.cls == 1) {
        if (t.precision != 32 && t.precision != 64) return fail(HPD_ERR_UNSUPPORTED, "Unsupported floating point precision");
        *dtype = t.precision == 32 ? HPD_F32 : HPD_F64;
        return HPD_OK;
    }
    return fail(HPD_ERR_UNSUPPORTED, "Unsupported data set type");
}

// ------------------------------------------------------------------ writing

// Raised for a file feature the writer does not handle (libhdf5 would).
struct Unsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

std::vector<unsigned char> entry_bytes(uint64_t name_off, uint64_t header) {
    std::vector<unsigned char> e(kSnodEntry, 0);  // cache type 0, empty scratch pad
    wr(&e[0], name_off, 8);
    wr(&e[8], header, 8);
    return e;
}

// Object header (version 1) of a 1-D little-endian int64 dataset of n elements stored
// contiguously at data_addr: dataspace, datatype, fill value and layout messages.
std::vector<unsigned char> labels_header(uint64_t n, uint64_t data_addr) {
    std::vector<unsigned char> h(16, 0);
    int nmsg = 0;
    auto msg = [&](int type, int flags, const std::vector<unsigned char>& body) {
        const uint64_t padded = (body.size() + 7) & ~7ull;
        const size_t at = h.size();
        h.resize(at + 8 + padded, 0);
        wr(&h[at], type, 2);
        wr(&h[at + 2], padded, 2);
        h[at + 4] = (unsigned char)flags;
        std::copy(body.begin(), body.end(), h.begin() + at + 8);
        ++nmsg;
    };
    std::vector<unsigned char> space(24, 0);  // version 1, rank 1, maximum dimensions present
    space[0] = 1;
    space[1] = 1;
    space[2] = 1;
    wr(&space[8], n, 8);
    wr(&space[16], n, 8);
    msg(0x01, 0, space);
    std::vector<unsigned char> type(12, 0);  // version 1 fixed-point: little-endian, signed, 8 bytes, 64 bits
    type[0] = 0x10;
    type[1] = 0x08;
    wr(&type[4], 8, 4);
    wr(&type[10], 64, 2);
    msg(0x03, 1, type);
    msg(0x05, 1, {2, 2, 2, 0});  // fill value version 2: allocation late, written if set, none defined
    std::vector<unsigned char> layout(18, 0);  // version 3 contiguous: address, size
    layout[0] = 3;
    layout[1] = 1;
    wr(&layout[2], n ? data_addr : kUndef, 8);
    wr(&layout[10], n * 8, 8);
    msg(0x08, 0, layout);
    h[0] = 1;
    wr(&h[2], nmsg, 2);
    wr(&h[4], 1, 4);
    wr(&h[8], h.size() - 16, 4);
    return h;
}

// A new file holding one root-level dataset of labels: superblock version 0, root group
// as a symbol table (B-tree, local heap, one symbol table node), the earliest format.
std::vector<unsigned char> new_file(const std::string& name, const int64_t* labels, uint64_t n) {
    constexpr int kLeafK = 4, kInternalK = 16;
    constexpr uint64_t sb = 0, root = 96, btree = root + 40;
    constexpr uint64_t btree_size = 24 + 2 * kInternalK * 8 + (2 * kInternalK + 1) * 8;
    const uint64_t heap = btree + btree_size, heap_data = heap + 32;
    const uint64_t name_bytes = (name.size() + 1 + 7) & ~7ull;
    const uint64_t heap_size = 8 + name_bytes;
    const uint64_t snod = heap_data + heap_size, snod_size = 8 + 2 * kLeafK * kSnodEntry;
    const uint64_t dset = snod + snod_size;
    const uint64_t dset_size = labels_header(n, 0).size();
    const uint64_t data = dset + dset_size, eof = data + n * 8;
    std::vector<unsigned char> b(eof, 0);
    std::memcpy(&b[sb], kSig, 8);
    b[sb + 13] = 8;  // size of offsets
    b[sb + 14] = 8;  // size of lengths
    wr(&b[sb + 16], kLeafK, 2);
    wr(&b[sb + 18], kInternalK, 2);
    wr(&b[sb + 32], kUndef, 8);  // free-space information
    wr(&b[sb + 40], eof, 8);
    wr(&b[sb + 48], kUndef, 8);  // driver information
    wr(&b[sb + 64], root, 8);    // root entry: header, cache type 1 (symbol table), B-tree, heap
    wr(&b[sb + 72], 1, 4);
    wr(&b[sb + 80], btree, 8);
    wr(&b[sb + 88], heap, 8);
    b[root] = 1;  // root object header: one symbol table message
    wr(&b[root + 2], 1, 2);
    wr(&b[root + 4], 1, 4);
    wr(&b[root + 8], 24, 4);
    wr(&b[root + 16], 0x11, 2);
    wr(&b[root + 18], 16, 2);
    wr(&b[root + 24], btree, 8);
    wr(&b[root + 32], heap, 8);
    std::memcpy(&b[btree], "TREE", 4);  // group node, level 0, one child
    wr(&b[btree + 6], 1, 2);
    wr(&b[btree + 8], kUndef, 8);
    wr(&b[btree + 16], kUndef, 8);
    wr(&b[btree + 24], 0, 8);
    wr(&b[btree + 32], snod, 8);
    wr(&b[btree + 40], 8, 8);
    std::memcpy(&b[heap], "HEAP", 4);  // local heap: "" at 0, the name at 8, no free block
    wr(&b[heap + 8], heap_size, 8);
    wr(&b[heap + 16], 1, 8);  // the format's end of the free list
    wr(&b[heap + 24], heap_data, 8);
    std::memcpy(&b[heap_data + 8], name.data(), name.size());
    std::memcpy(&b[snod], "SNOD", 4);
    b[snod + 4] = 1;
    wr(&b[snod + 6], 1, 2);
    const std::vector<unsigned char> e = entry_bytes(8, dset);
    std::copy(e.begin(), e.end(), b.begin() + snod + 8);
    const std::vector<unsigned char> h = labels_header(n, data);
    std::copy(h.begin(), h.end(), b.begin() + dset);
    for (uint64_t i = 0; i < n; ++i) wr(&b[data + 8 * i], (uint64_t)labels[i], 8);
    return b;
}

// Links `name` -> `header` into a symbol-table group whose B-tree is a single leaf-level
// node: the name is appended to the local heap (its data segment moved to the end of
// the file), the entry inserted in name order, a full symbol table node split in two.
void insert_link(File& f, uint64_t group, const std::string& name, uint64_t header) {
    const SymTab st = symbol_table(f, group);
    if (st.btree == kUndef) throw Unsupported("adding to a group held as link messages");
    Heap hp = local_heap(f, st.heap);
    const uint64_t name_bytes = (name.size() + 1 + 7) & ~7ull;
    const uint64_t grown = hp.size + name_bytes;
    const uint64_t seg = f.alloc(grown);
    std::memcpy(f.ptr(seg, grown), f.at(hp.data, hp.size), hp.size);
    std::memcpy(f.ptr(seg + hp.size, name_bytes), name.data(), name.size());
    const uint64_t name_off = hp.size;
    unsigned char* hh = f.mut(st.heap, 32);
    wr(hh + 8, grown, 8);
    wr(hh + 24, seg, 8);
    hp = {st.heap, seg, grown};

    const unsigned char* t = f.at(st.btree, 24);
    if (std::memcmp(t, "TREE", 4) != 0 || t[4] != 0) throw Bad("bad group B-tree node");
    if (t[5] != 0) throw Unsupported("adding to a group B-tree of more than one level");
    const uint64_t cap = 2 * (uint64_t)f.internal_k, leaf_cap = 2 * (uint64_t)f.leaf_k;
    const uint64_t used = rd(t + 6, 2);
    if (used > cap) throw Bad("bad group B-tree node");
    std::vector<uint64_t> keys(used + 1), kids(used);
    const unsigned char* kc = f.at(st.btree + 24, (2 * used + 1) * 8);
    for (uint64_t i = 0; i <= used; ++i) keys[i] = rd(kc + 16 * i, 8);
    for (uint64_t i = 0; i < used; ++i) kids[i] = rd(kc + 16 * i + 8, 8);
    const std::vector<unsigned char> entry = entry_bytes(name_off, header);
    auto new_snod = [&](const std::vector<std::vector<unsigned char>>& es) {
        const uint64_t a = f.alloc(8 + leaf_cap * kSnodEntry);
        unsigned char* s = f.ptr(a, 8 + es.size() * kSnodEntry);
        std::memcpy(s, "SNOD", 4);
        s[4] = 1;
        wr(s + 6, es.size(), 2);
        for (size_t k = 0; k < es.size(); ++k) std::memcpy(s + 8 + k * kSnodEntry, es[k].data(), kSnodEntry);
        return a;
    };
    if (used == 0) {
        kids = {new_snod({entry})};
        keys = {0, name_off};
    } else {
        uint64_t i = 0;
        while (i < used && name.compare(heap_name(f, hp, keys[i + 1])) > 0) ++i;
        const bool last = i == used;
        if (last) i = used - 1;
        const unsigned char* s = f.at(kids[i], 8);
        if (std::memcmp(s, "SNOD", 4) != 0) throw Bad("bad symbol table node");
        const uint64_t n = rd(s + 6, 2);
        if (n > leaf_cap) throw Bad("bad symbol table node");
        std::vector<std::vector<unsigned char>> es;
        const unsigned char* e = f.at(kids[i] + 8, n * kSnodEntry);
        for (uint64_t k = 0; k < n; ++k) es.emplace_back(e + k * kSnodEntry, e + (k + 1) * kSnodEntry);
        size_t j = 0;
        while (j < es.size() && name.compare(heap_name(f, hp, rd(es[j].data(), 8))) > 0) ++j;
        es.insert(es.begin() + j, entry);
        if (es.size() <= leaf_cap) {
            unsigned char* w = f.mut(kids[i], 8 + es.size() * kSnodEntry);
            wr(w + 6, es.size(), 2);
            for (size_t k = 0; k < es.size(); ++k) std::memcpy(w + 8 + k * kSnodEntry, es[k].data(), kSnodEntry);
        } else {
            if (used == cap) throw Unsupported("adding to a full group B-tree node");
            const size_t left = (es.size() + 1) / 2;
            const std::vector<std::vector<unsigned char>> right(es.begin() + left, es.end());
            unsigned char* w = f.mut(kids[i], 8 + left * kSnodEntry);
            wr(w + 6, left, 2);
            for (size_t k = 0; k < left; ++k) std::memcpy(w + 8 + k * kSnodEntry, es[k].data(), kSnodEntry);
            const uint64_t a = new_snod(right);
            kids.insert(kids.begin() + i + 1, a);
            keys.insert(keys.begin() + i + 1, rd(es[left - 1].data(), 8));
        }
        if (last) keys.back() = name_off;
    }
    const uint64_t now = kids.size();
    unsigned char* w = f.mut(st.btree, 24 + (2 * now + 1) * 8);
    wr(w + 6, now, 2);
    for (uint64_t i = 0; i <= now; ++i) wr(w + 24 + 16 * i, keys[i], 8);
    for (uint64_t i = 0; i < now; ++i) wr(w + 32 + 16 * i, kids[i], 8);
}

// The reference writes H5T_NATIVE_LONG values; libhdf5 converts them to the dataset's
// type, integers saturating at the type's range, floating point rounding to nearest.
std::vector<unsigned char> convert_labels(const Dtype& t, const int64_t* labels, uint64_t m) {
    std::vector<unsigned char> out(m * t.size);
    if (t.cls == 0 && t.offset == 0 && t.precision == (int)t.size * 8 &&
        (t.size == 1 || t.size == 2 || t.size == 4 || t.size == 8)) {
        const int bits = t.precision;
        for (uint64_t i = 0; i < m; ++i) {
            const int64_t v = labels[i];
            uint64_t u;
            if (t.sign) {
                const int64_t hi = bits == 64 ? INT64_MAX : (int64_t(1) << (bits - 1)) - 1;
                const int64_t lo = bits == 64 ? INT64_MIN : -(int64_t(1) << (bits - 1));
                u = (uint64_t)std::min(std::max(v, lo), hi);
            } else {
                const uint64_t hi = bits == 64 ? UINT64_MAX : (uint64_t(1) << bits) - 1;
                u = v < 0 ? 0 : std::min((uint64_t)v, hi);
            }
            wr(&out[i * t.size], u, (int)t.size);
        }
    } else if (t.cls == 1 && t.ieee) {
        for (uint64_t i = 0; i < m; ++i) {
            if (t.size == 4) {
                const float x = (float)labels[i];
                std::memcpy(&out[i * 4], &x, 4);
            } else {
                const double x = (double)labels[i];
                std::memcpy(&out[i * 8], &x, 8);
            }
        }
    } else {
        throw Bad("no conversion from int64 to the dataset's element type");
    }
    if (t.big) swap_bytes(out.data(), m, t.size);
    return out;
}

// Writes the first n elements of an existing dataset as the reference's H5Dwrite does:
// a 1-D dataset of at least n elements, or any dataset of exactly n elements.
void write_into(File& f, const Dataset& ds, const int64_t* labels, uint64_t n) {
    uint64_t total = 1;
    for (uint64_t d : ds.dims)
        if (!mul_ok(total, d, total)) throw Bad("dataset extent overflows");
    if (!((ds.rank == 1 && ds.dims[0] >= n) || total == n)) throw Bad("extent differs from the labels");
    const std::vector<unsigned char> bytes = convert_labels(ds.type, labels, n);
    if (n == 0) return;
    const bool v1_header = std::memcmp(f.at(ds.header, 4), "OHDR", 4) != 0;
    if (ds.filtered || ds.external) throw Unsupported("writing filtered or external datasets");
    if (ds.layout_class == 1) {
        uint64_t data = ds.data;
        if (data == kUndef) {  // storage never allocated: allocate it and record it in the layout message
            if (!v1_header) throw Unsupported("allocating storage behind a checksummed object header");
            const uint64_t full = total * ds.type.size;
            data = f.alloc(full);
            unsigned char* d = f.ptr(data, full);
            if (ds.fill.size() == ds.type.size)
                for (uint64_t i = 0; i < total; ++i) std::memcpy(d + i * ds.type.size, ds.fill.data(), ds.type.size);
            wr(f.mut(ds.layout_msg + (ds.layout_version == 3 ? 2 : 8), 8), data, 8);
        } else if (ds.data_size < bytes.size()) {
            throw Bad("dataset storage smaller than its extent");
        }
        if (!bytes.empty()) std::memcpy(f.mut(data, bytes.size()), bytes.data(), bytes.size());
        return;
    }
    if (ds.layout_class == 0) {
        if (!v1_header) throw Unsupported("compact data inside a checksummed object header");
        if (ds.data_size < bytes.size()) throw Bad("dataset storage smaller than its extent");
        if (!bytes.empty()) std::memcpy(f.mut(ds.data, bytes.size()), bytes.data(), bytes.size());
        return;
    }
    throw Unsupported("writing chunked datasets");
}

// pwrite of the whole range (regular files may still return short counts).
bool write_at(int fd, const unsigned char* p, uint64_t n, uint64_t at) {
    while (n > 0) {
        const ssize_t w = pwrite(fd, p, n, (off_t)at);
        if (w <= 0) return false;
        p += w;
        n -= (uint64_t)w;
        at += (uint64_t)w;
    }
    return true;
}

// Writes the modified ranges and the appended bytes back, with the new end-of-file address.
void flush(File& f, const std::string& path) {
    if (!f.tail.empty()) {
        if (f.sb_version > 1) throw Unsupported("growing a file with a checksummed superblock");
        wr(f.mut(f.sb + 40 + (f.sb_version == 1 ? 4 : 0) - f.base, 8), f.end(), 8);
    }
    const int fd = open(path.c_str(), O_WRONLY);
    if (fd < 0) throw Bad("cannot reopen the file for writing");
    bool ok = true;
    for (const auto& r : f.dirty) ok = ok && write_at(fd, f.map + r.first, r.second - r.first, r.first);
    if (!f.tail.empty()) ok = ok && write_at(fd, f.tail.data(), f.tail.size(), f.size);
    ok = close(fd) == 0 && ok;
    if (!ok) throw Bad("short write");
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

int hpd_h5_read(const char* path, const char* dataset, void** data, int64_t* n, int32_t* d, int32_t* dtype) {
    if (!path || !dataset || !data || !n || !d || !dtype) return fail(HPD_ERR_INVALID, "null argument");
    *data = nullptr;
    const std::string p(path), name(dataset);
    File f;
    try {
        if (!open_file(p, f, false)) return fail(HPD_ERR_INVALID, "Could not open " + p);
    } catch (const std::exception& e) {
        return fail(HPD_ERR_INVALID, why(("Could not open " + p).c_str(), e));
    }
    Dataset ds;
    try {
        const uint64_t obj = find_object(f, split_path(name));
        if (obj == kUndef) return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
        ds = parse_dataset(f, obj);
        if (!ds.has_layout) return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
    } catch (const std::exception& e) {
        return fail(HPD_ERR_INVALID, why(("Could not open dataset " + name).c_str(), e));
    }
    if (!ds.has_type) return fail(HPD_ERR_RUNTIME, "Could not retrieve dataset type");
    if (ds.rank < 0) return fail(HPD_ERR_RUNTIME, "Could not retrieve dataspace extent, file seems to be corrupted");
    if (ds.rank != 2) return fail(HPD_ERR_INVALID, "Data in dataset " + name + " should be a matrix");
    int32_t ty = 0;
    if (const int rc = dtype_of(ds.type, &ty)) return rc;
    if (ds.type.cls == 0 && (ds.type.offset != 0 || (int)ds.type.size * 8 != ds.type.precision))
        return fail(HPD_ERR_RUNTIME, "Failed to read data (integers with padding bits)");
    if (ds.type.cls == 1 && !ds.type.ieee)
        return fail(HPD_ERR_RUNTIME, "Failed to read data (a floating-point layout other than IEEE 754)");
    uint64_t count, bytes;
    if (!mul_ok(ds.dims[0], ds.dims[1], count) || !mul_ok(count, ds.type.size, bytes) || ds.dims[0] > INT64_MAX ||
        ds.dims[1] > INT32_MAX)
        return fail(HPD_ERR_RUNTIME, "Failed to read data (extent too large)");
    void* buf = std::malloc(bytes ? bytes : 1);
    if (!buf) return fail(HPD_ERR_NOMEM, "Failed to read data (out of host memory)");
    try {
        read_elements(f, ds, static_cast<unsigned char*>(buf), count);
    } catch (const std::exception& e) {
        std::free(buf);
        return fail(HPD_ERR_RUNTIME, why("Failed to read data", e));
    }
    if (ds.type.big && ds.type.size > 1) swap_bytes(static_cast<unsigned char*>(buf), count, ds.type.size);
    *data = buf;
    *n = (int64_t)ds.dims[0];
    *d = (int32_t)ds.dims[1];
    *dtype = ty;
    return HPD_OK;
}

void hpd_h5_free(void* data) { std::free(data); }

int hpd_h5_write(const char* path, const char* dataset, const int64_t* labels, int64_t n) {
    if (!path || !dataset || (n > 0 && !labels) || n < 0) return fail(HPD_ERR_INVALID, "null argument or negative size");
    const std::string p(path), name(dataset);
    const std::vector<std::string> parts = split_path(name);
    // H5Fcreate(H5F_ACC_EXCL) first: a file that does not exist yet is created with the dataset
    const int fd = open(p.c_str(), O_WRONLY | O_CREAT | O_EXCL, 0644);
    if (fd >= 0) {
        if (parts.size() != 1) {
            close(fd);
            return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
        }
        const std::vector<unsigned char> b = new_file(parts[0], labels, (uint64_t)n);
        const bool ok = write_at(fd, b.data(), b.size(), 0);
        if (close(fd) != 0 || !ok)
            return fail(HPD_ERR_RUNTIME, "Failed to write data, target data set is probably of wrong size or type");
        return HPD_OK;
    }
    File f;
    try {
        if (!open_file(p, f, true) || access(p.c_str(), W_OK) != 0) return fail(HPD_ERR_INVALID, "Could not open " + p);
    } catch (const std::exception& e) {
        return fail(HPD_ERR_INVALID, why(("Could not open " + p).c_str(), e));
    }
    if (parts.empty()) return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
    Dataset ds;
    try {
        const std::vector<std::string> parent(parts.begin(), parts.end() - 1);
        const uint64_t group = find_object(f, parent);
        if (group == kUndef) return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
        uint64_t obj = child_of(f, group, parts.back());
        if (obj == kUndef) {  // H5Dcreate1: a new 1-D int64 dataset in the group
            if (f.sb_version > 1) throw Unsupported("adding a dataset to a file with a checksummed superblock");
            const uint64_t hdr_size = labels_header((uint64_t)n, 0).size();
            obj = f.alloc(hdr_size);
            const uint64_t data = n ? f.alloc((uint64_t)n * 8) : kUndef;
            const std::vector<unsigned char> h = labels_header((uint64_t)n, data);
            std::memcpy(f.ptr(obj, h.size()), h.data(), h.size());
            insert_link(f, group, parts.back(), obj);
        }
        ds = parse_dataset(f, obj);
        if (!is_dataset(ds)) return fail(HPD_ERR_INVALID, "Could not open dataset " + name);
    } catch (const std::exception& e) {
        return fail(HPD_ERR_INVALID, why(("Could not open dataset " + name).c_str(), e));
    }
    try {
        write_into(f, ds, labels, (uint64_t)n);
        flush(f, p);
    } catch (const std::exception& e) {
        return fail(HPD_ERR_RUNTIME, why("Failed to write data, target data set is probably of wrong size or type", e));
    }
    return HPD_OK;
}

}  // extern "C"
