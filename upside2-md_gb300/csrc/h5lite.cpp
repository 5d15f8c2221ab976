// h5lite reader implementation.  Format facts follow the public "HDF5 File
// Format Specification" (superblock v0/v1, object header v1, v1 B-trees,
// local heaps, symbol-table nodes, messages 0x1/0x3/0x8/0xB/0xC/0x10/0x11).
#include "h5lite.h"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>

namespace h5lite {

// ---------------------------------------------------------------- inflate ---
namespace {

struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    int bits(int need) {
        uint32_t val = bitbuf;
        while (bitcnt < need) {
            if (pos >= n) throw Error("deflate stream truncated");
            val |= uint32_t(p[pos++]) << bitcnt;
            bitcnt += 8;
        }
        bitbuf = val >> need;
        bitcnt -= need;
        return int(val & ((1u << need) - 1u));
    }
};

struct Huff {
    short count[16];
    short symbol[320];
};

// Canonical Huffman table from code lengths (RFC 1951 section 3.2.2).
void build_huff(Huff& h, const short* length, int n) {
    for (int i = 0; i < 16; ++i) h.count[i] = 0;
    for (int s = 0; s < n; ++s) h.count[length[s]]++;
    short offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = short(offs[len] + h.count[len]);
    for (int s = 0; s < n; ++s)
        if (length[s]) h.symbol[offs[length[s]]++] = short(s);
}

int huff_decode(BitIn& s, const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len <= 15; ++len) {
        code |= s.bits(1);
        int count = h.count[len];
        if (code - count < first) return h.symbol[index + (code - first)];
        index += count;
        first += count;
        first <<= 1;
        code <<= 1;
    }
    throw Error("invalid Huffman code in deflate stream");
}

const short kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                            31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const short kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                             2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const short kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                             193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                             6145, 8193, 12289, 16385, 24577};
const short kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                              6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_codes(BitIn& s, std::vector<uint8_t>& out, const Huff& lencode, const Huff& distcode) {
    for (;;) {
        int sym = huff_decode(s, lencode);
        if (sym < 256) {
            out.push_back(uint8_t(sym));
        } else if (sym == 256) {
            return;
        } else {
            sym -= 257;
            if (sym >= 29) throw Error("bad length symbol in deflate stream");
            int len = kLenBase[sym] + s.bits(kLenExtra[sym]);
            int dsym = huff_decode(s, distcode);
            if (dsym >= 30) throw Error("bad distance symbol in deflate stream");
            size_t dist = size_t(kDistBase[dsym] + s.bits(kDistExtra[dsym]));
            if (dist > out.size()) throw Error("deflate distance too far back");
            size_t from = out.size() - dist;
            for (int i = 0; i < len; ++i) out.push_back(out[from + i]);
        }
    }
}

}  // namespace

std::vector<uint8_t> inflate_zlib(const uint8_t* src, size_t n, size_t size_hint) {
    if (n < 2) throw Error("zlib stream too short");
    int cmf = src[0], flg = src[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0) throw Error("bad zlib header");
    if (flg & 32) throw Error("zlib preset dictionary unsupported");
    BitIn s{src + 2, n - 2};
    std::vector<uint8_t> out;
    out.reserve(size_hint);
    int last;
    do {
        last = s.bits(1);
        int type = s.bits(2);
        if (type == 0) {
            s.bitbuf = 0;
            s.bitcnt = 0;
            if (s.pos + 4 > s.n) throw Error("stored block truncated");
            unsigned len = s.p[s.pos] | (s.p[s.pos + 1] << 8);
            unsigned nlen = s.p[s.pos + 2] | (s.p[s.pos + 3] << 8);
            s.pos += 4;
            if (len != (~nlen & 0xffffu)) throw Error("stored block length mismatch");
            if (s.pos + len > s.n) throw Error("stored block truncated");
            out.insert(out.end(), s.p + s.pos, s.p + s.pos + len);
            s.pos += len;
        } else if (type == 1) {
            static Huff fl, fd;
            static bool init = false;
            if (!init) {
                short lengths[288];
                int i = 0;
                for (; i < 144; ++i) lengths[i] = 8;
                for (; i < 256; ++i) lengths[i] = 9;
                for (; i < 280; ++i) lengths[i] = 7;
                for (; i < 288; ++i) lengths[i] = 8;
                build_huff(fl, lengths, 288);
                for (i = 0; i < 30; ++i) lengths[i] = 5;
                build_huff(fd, lengths, 30);
                init = true;
            }
            inflate_codes(s, out, fl, fd);
        } else if (type == 2) {
            static const short order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            int nlen = s.bits(5) + 257, ndist = s.bits(5) + 1, ncode = s.bits(4) + 4;
            if (nlen > 286 || ndist > 30) throw Error("bad dynamic block counts");
            short lengths[320];
            int idx;
            for (idx = 0; idx < ncode; ++idx) lengths[order[idx]] = short(s.bits(3));
            for (; idx < 19; ++idx) lengths[order[idx]] = 0;
            Huff lencode, distcode;
            build_huff(lencode, lengths, 19);
            idx = 0;
            while (idx < nlen + ndist) {
                int sym = huff_decode(s, lencode);
                if (sym < 16) {
                    lengths[idx++] = short(sym);
                } else {
                    short len = 0;
                    int rep;
                    if (sym == 16) {
                        if (idx == 0) throw Error("repeat with no previous length");
                        len = lengths[idx - 1];
                        rep = 3 + s.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + s.bits(3);
                    } else {
                        rep = 11 + s.bits(7);
                    }
                    if (idx + rep > nlen + ndist) throw Error("too many code lengths");
                    while (rep--) lengths[idx++] = len;
                }
            }
            build_huff(lencode, lengths, nlen);
            build_huff(distcode, lengths + nlen, ndist);
            inflate_codes(s, out, lencode, distcode);
        } else {
            throw Error("invalid deflate block type");
        }
    } while (!last);
    return out;
}

// ----------------------------------------------------------- file parsing ---
namespace {
inline uint64_t rd(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}
constexpr uint64_t UNDEF = ~uint64_t(0);
}  // namespace

File::File(const std::string& path) : fname_(path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error("cannot open HDF5 file '" + path + "'");
    f.seekg(0, std::ios::end);
    size_t sz = size_t(f.tellg());
    f.seekg(0);
    buf_.resize(sz);
    if (sz) f.read(reinterpret_cast<char*>(buf_.data()), std::streamsize(sz));
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    // The superblock may sit at 0, 512, 1024, ... (user block)
    size_t sb = UNDEF;
    for (size_t off = 0; off + 8 <= sz; off = off ? off * 2 : 512) {
        if (!memcmp(buf_.data() + off, sig, 8)) { sb = off; break; }
    }
    if (sb == size_t(UNDEF)) throw Error("'" + path + "' is not an HDF5 file");
    const uint8_t* p = at(sb, 96);
    int version = p[8];
    if (version > 1) throw Error("HDF5 superblock version " + std::to_string(version) + " unsupported");
    if (p[13] != 8 || p[14] != 8) throw Error("only 8-byte offsets/lengths supported");
    size_t q = sb + 24 + (version == 1 ? 4 : 0);
    base_ = rd(at(q, 8), 8);
    q += 32;  // base, free-space, eof, driver
    // root group symbol table entry: link name offset, object header address
    root_addr_ = rd(at(q + 8, 8), 8);
}

File::~File() = default;

const uint8_t* File::at(uint64_t addr, size_t n) const {
    if (addr == UNDEF || addr + n > buf_.size() || addr + n < addr)
        throw Error("HDF5 address out of range in '" + fname_ + "'");
    return buf_.data() + addr;
}

Object& File::load(uint64_t addr) {
    auto it = cache_.find(addr);
    if (it != cache_.end()) return *it->second;
    auto obj = std::make_unique<Object>();
    obj->addr = addr;
    parse_header(*obj);
    Object& ref = *obj;
    cache_[addr] = std::move(obj);
    return ref;
}

void File::parse_header(Object& obj) {
    const uint8_t* h = at(base_ + obj.addr, 16);
    if (h[0] != 1) throw Error("object header version " + std::to_string(h[0]) + " unsupported (only v1)");
    int n_msg = int(rd(h + 2, 2));
    uint64_t hsize = rd(h + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{base_ + obj.addr + 16, hsize}};
    int seen = 0;
    for (size_t bi = 0; bi < blocks.size() && seen < n_msg; ++bi) {
        uint64_t pos = blocks[bi].first, end = blocks[bi].first + blocks[bi].second;
        while (pos + 8 <= end && seen < n_msg) {
            const uint8_t* m = at(pos, 8);
            int type = int(rd(m, 2));
            size_t size = size_t(rd(m + 2, 2));
            const uint8_t* data = at(pos + 8, size);
            ++seen;
            if (type == 0x10) {
                blocks.push_back({base_ + rd(data, 8), rd(data + 8, 8)});
            } else {
                parse_message(obj, type, data, size);
            }
            pos += 8 + size;
        }
    }
}

namespace {
Dtype parse_dtype(const uint8_t* p) {
    Dtype dt;
    int cls = p[0] & 15;
    dt.size = int(rd(p + 4, 4));
    if (cls == 0) {
        dt.cls = DT_INT;
        dt.big_endian = p[1] & 1;
        dt.is_signed = (p[1] >> 3) & 1;
    } else if (cls == 1) {
        dt.cls = DT_FLOAT;
        dt.big_endian = p[1] & 1;
        dt.is_signed = true;
    } else if (cls == 3) {
        dt.cls = DT_STRING;
    } else {
        dt.cls = DT_OTHER;
    }
    return dt;
}

// Returns dims; sets scalar when rank 0.
std::vector<uint64_t> parse_dataspace(const uint8_t* p, bool* scalar, bool* null_space = nullptr) {
    int version = p[0];
    int rank = p[1];
    int flags = p[2];
    const uint8_t* d;
    if (version == 1) {
        d = p + 8;
        *scalar = (rank == 0);
    } else if (version == 2) {
        d = p + 4;
        *scalar = (p[3] == 0);
        if (null_space) *null_space = (p[3] == 2);
    } else {
        throw Error("dataspace version unsupported");
    }
    (void)flags;
    std::vector<uint64_t> dims(static_cast<size_t>(rank));
    for (int i = 0; i < rank; ++i) dims[i] = rd(d + 8 * i, 8);
    return dims;
}
}  // namespace

void File::parse_message(Object& obj, int type, const uint8_t* p, size_t n) {
    switch (type) {
        case 0x0001: obj.dims = parse_dataspace(p, &obj.is_scalar); break;
        case 0x0003:
            obj.dt = parse_dtype(p);
            obj.dt.raw.assign(p, p + n);
            break;
        case 0x0008: {
            int version = p[0];
            if (version == 3) {
                obj.layout_class = p[1];
                if (obj.layout_class == 0) {
                    size_t sz = size_t(rd(p + 2, 2));
                    obj.compact_data.assign(p + 4, p + 4 + sz);
                } else if (obj.layout_class == 1) {
                    obj.data_addr = rd(p + 2, 8);
                    obj.data_size = rd(p + 10, 8);
                } else if (obj.layout_class == 2) {
                    int rank = p[2];
                    obj.data_addr = rd(p + 3, 8);
                    obj.chunk_dims.resize(size_t(rank));
                    for (int i = 0; i < rank; ++i) obj.chunk_dims[i] = uint32_t(rd(p + 11 + 4 * i, 4));
                } else {
                    throw Error("unsupported layout class");
                }
            } else if (version == 1 || version == 2) {
                int rank = p[1];
                obj.layout_class = p[2];
                const uint8_t* q = p + 8;
                if (obj.layout_class != 0) { obj.data_addr = rd(q, 8); q += 8; }
                std::vector<uint32_t> dims(static_cast<size_t>(rank));
                for (int i = 0; i < rank; ++i) dims[i] = uint32_t(rd(q + 4 * i, 4));
                q += 4 * rank;
                if (obj.layout_class == 2) {
                    obj.chunk_dims = dims;
                } else if (obj.layout_class == 0) {
                    size_t sz = size_t(rd(q, 4));
                    obj.compact_data.assign(q + 4, q + 4 + sz);
                } else {
                    uint64_t total = 1;
                    for (int i = 0; i < rank; ++i) total *= dims[i];
                    obj.data_size = total;  // element count * elem size provided by dims
                }
            } else {
                throw Error("unsupported layout message version");
            }
            break;
        }
        case 0x000B: {
            int version = p[0], nf = p[1];
            const uint8_t* q = p + (version == 1 ? 8 : 2);
            for (int i = 0; i < nf; ++i) {
                int id = int(rd(q, 2));
                int name_len = 0;
                if (version == 1 || id >= 256) { name_len = int(rd(q + 2, 2)); q += 2; }
                int ncd = int(rd(q + 4, 2));
                q += 6;
                if (version == 1) name_len = (name_len + 7) & ~7;
                q += name_len;
                q += 4 * ncd;
                if (version == 1 && (ncd & 1)) q += 4;
                obj.filters.push_back(id);
            }
            break;
        }
        case 0x000C: {
            Attribute a;
            int version = p[0];
            size_t name_sz = size_t(rd(p + 2, 2)), dt_sz = size_t(rd(p + 4, 2)), ds_sz = size_t(rd(p + 6, 2));
            const uint8_t* q = p + (version == 3 ? 9 : 8);
            auto pad = [&](size_t s) { return version == 1 ? ((s + 7) & ~size_t(7)) : s; };
            a.name.assign(reinterpret_cast<const char*>(q), strnlen(reinterpret_cast<const char*>(q), name_sz));
            q += pad(name_sz);
            a.dt = parse_dtype(q);
            a.dt.raw.assign(q, q + dt_sz);
            q += pad(dt_sz);
            bool scalar, null_space = false;
            a.dims = parse_dataspace(q, &scalar, &null_space);
            q += pad(ds_sz);
            uint64_t cnt = null_space ? 0 : 1;
            for (auto d : a.dims) cnt *= d;
            size_t nbytes = size_t(cnt) * size_t(a.dt.size);
            if (q + nbytes > p + n) throw Error("attribute '" + a.name + "' data overruns its message");
            a.data.assign(q, q + nbytes);
            obj.attrs.push_back(std::move(a));
            break;
        }
        case 0x0011: {
            obj.is_group = true;
            uint64_t btree = rd(p, 8), heap = rd(p + 8, 8);
            const uint8_t* hp = at(base_ + heap, 32);
            if (memcmp(hp, "HEAP", 4)) throw Error("bad local heap signature");
            uint64_t heap_data = rd(hp + 24, 8);
            read_group_btree(btree, heap_data, obj.links);
            break;
        }
        case 0x0006:
        case 0x0002:
            throw Error("new-style (link message) groups are not supported");
        default: break;  // fill value, modification time, etc.
    }
}

void File::read_group_btree(uint64_t btree_addr, uint64_t heap_data,
                            std::vector<std::pair<std::string, uint64_t>>& out) {
    const uint8_t* b = at(base_ + btree_addr, 24);
    if (memcmp(b, "TREE", 4)) throw Error("bad group B-tree signature");
    int level = b[5];
    int used = int(rd(b + 6, 2));
    const uint8_t* e = at(base_ + btree_addr + 24, size_t(used) * 16 + 8);
    for (int i = 0; i < used; ++i) {
        uint64_t child = rd(e + 8 + 16 * i, 8);
        if (level > 0) {
            read_group_btree(child, heap_data, out);
        } else {
            const uint8_t* s = at(base_ + child, 8);
            if (memcmp(s, "SNOD", 4)) throw Error("bad symbol node signature");
            int nsym = int(rd(s + 6, 2));
            const uint8_t* ent = at(base_ + child + 8, size_t(nsym) * 40);
            for (int k = 0; k < nsym; ++k) {
                uint64_t name_off = rd(ent + 40 * k, 8);
                uint64_t oh = rd(ent + 40 * k + 8, 8);
                const char* nm = reinterpret_cast<const char*>(at(base_ + heap_data + name_off, 1));
                size_t maxlen = buf_.size() - size_t(base_ + heap_data + name_off);
                out.emplace_back(std::string(nm, strnlen(nm, maxlen)), oh);
            }
        }
    }
}

Object& File::resolve(const std::string& path) {
    Object* cur = &load(root_addr_);
    std::stringstream ss(path);
    std::string part;
    while (std::getline(ss, part, '/')) {
        if (part.empty() || part == ".") continue;
        if (!cur->is_group) throw Error("'" + path + "': intermediate object is not a group");
        uint64_t next = UNDEF;
        for (auto& kv : cur->links)
            if (kv.first == part) { next = kv.second; break; }
        if (next == UNDEF) throw Error("'" + path + "' not found in '" + fname_ + "'");
        cur = &load(next);
    }
    return *cur;
}

bool File::exists(const std::string& path) {
    try { resolve(path); return true; } catch (const Error&) { return false; }
}

bool File::is_group(const std::string& path) { return resolve(path).is_group; }

std::vector<std::string> File::list(const std::string& group_path) {
    Object& o = resolve(group_path);
    if (!o.is_group) throw Error("'" + group_path + "' is not a group");
    std::vector<std::string> names;
    for (auto& kv : o.links) names.push_back(kv.first);
    std::sort(names.begin(), names.end());
    return names;
}

std::vector<uint64_t> File::dims(const std::string& p) { return resolve(p).dims; }
Dtype File::dtype(const std::string& p) { return resolve(p).dt; }

void File::read_chunk_btree(const Object& obj, uint64_t addr, std::vector<uint8_t>& out) {
    const uint8_t* b = at(base_ + addr, 24);
    if (memcmp(b, "TREE", 4)) throw Error("bad chunk B-tree signature");
    if (b[4] != 1) throw Error("expected raw-data chunk B-tree");
    int level = b[5];
    int used = int(rd(b + 6, 2));
    size_t rank = obj.chunk_dims.size();  // includes element dim
    size_t key_sz = 8 + 8 * rank;
    const uint8_t* e = at(base_ + addr + 24, size_t(used) * (key_sz + 8) + key_sz);
    size_t esz = size_t(obj.dt.size);
    size_t nd = obj.dims.size();
    for (int i = 0; i < used; ++i) {
        const uint8_t* key = e + i * (key_sz + 8);
        uint64_t child = rd(key + key_sz, 8);
        if (level > 0) { read_chunk_btree(obj, child, out); continue; }
        uint32_t csize = uint32_t(rd(key, 4));
        uint32_t fmask = uint32_t(rd(key + 4, 4));
        std::vector<uint64_t> off(nd);
        for (size_t d = 0; d < nd; ++d) off[d] = rd(key + 8 + 8 * d, 8);
        size_t chunk_elems = 1;
        for (size_t d = 0; d < nd; ++d) chunk_elems *= obj.chunk_dims[d];
        size_t chunk_bytes = chunk_elems * esz;
        const uint8_t* raw = at(base_ + child, csize);
        std::vector<uint8_t> data(raw, raw + csize);
        for (int fi = int(obj.filters.size()) - 1; fi >= 0; --fi) {
            if (fmask & (1u << fi)) continue;
            int id = obj.filters[size_t(fi)];
            if (id == 3) {  // fletcher32: drop trailing checksum
                if (data.size() < 4) throw Error("fletcher32 chunk too small");
                data.resize(data.size() - 4);
            } else if (id == 1) {
                data = inflate_zlib(data.data(), data.size(), chunk_bytes);
            } else if (id == 2) {
                std::vector<uint8_t> un(data.size());
                size_t ne = data.size() / esz;
                for (size_t k = 0; k < esz; ++k)
                    for (size_t j = 0; j < ne; ++j) un[j * esz + k] = data[k * ne + j];
                // trailing bytes that do not form a whole element stay in place
                for (size_t j = ne * esz; j < data.size(); ++j) un[j] = data[j];
                data.swap(un);
            } else {
                throw Error("unsupported HDF5 filter id " + std::to_string(id));
            }
        }
        if (data.size() < chunk_bytes) throw Error("decoded chunk smaller than chunk shape");
        // scatter chunk into the dense row-major output, clipping at dataset bounds
        std::vector<uint64_t> idx(nd, 0);
        for (size_t k = 0; k < chunk_elems; ++k) {
            // decompose k into chunk coordinates (row-major)
            size_t rem = k;
            bool inside = true;
            uint64_t lin = 0;
            for (int d = int(nd) - 1; d >= 0; --d) {
                idx[size_t(d)] = rem % obj.chunk_dims[size_t(d)];
                rem /= obj.chunk_dims[size_t(d)];
            }
            for (size_t d = 0; d < nd; ++d) {
                uint64_t g = off[d] + idx[d];
                if (g >= obj.dims[d]) { inside = false; break; }
                lin = lin * obj.dims[d] + g;
            }
            if (inside) memcpy(out.data() + lin * esz, data.data() + k * esz, esz);
        }
    }
}

std::vector<uint8_t> File::read_raw(const std::string& path) {
    Object& o = resolve(path);
    if (o.is_group) throw Error("'" + path + "' is a group, not a dataset");
    uint64_t cnt = 1;
    for (auto d : o.dims) cnt *= d;
    size_t nbytes = size_t(cnt) * size_t(o.dt.size);
    std::vector<uint8_t> out(nbytes, 0);
    if (nbytes == 0) return out;
    if (o.layout_class == 0) {
        if (o.compact_data.size() < nbytes) throw Error("compact data too small");
        memcpy(out.data(), o.compact_data.data(), nbytes);
    } else if (o.layout_class == 1) {
        if (o.data_addr == UNDEF) return out;  // never written: fill with zeros
        memcpy(out.data(), at(base_ + o.data_addr, nbytes), nbytes);
    } else if (o.layout_class == 2) {
        if (o.data_addr != UNDEF) read_chunk_btree(o, o.data_addr, out);
    } else {
        throw Error("dataset '" + path + "' has no layout message");
    }
    return out;
}

void convert_elements(const Dtype& dt, const uint8_t* src, size_t n, int kind, void* dst) {
    for (size_t i = 0; i < n; ++i) {
        const uint8_t* s = src + i * size_t(dt.size);
        uint8_t tmp[8];
        if (dt.size > 8) throw Error("element too wide");
        if (dt.big_endian) {
            for (int k = 0; k < dt.size; ++k) tmp[k] = s[dt.size - 1 - k];
            s = tmp;
        }
        double dv = 0;
        int64_t iv = 0;
        bool is_int = dt.cls == DT_INT;
        if (dt.cls == DT_FLOAT) {
            if (dt.size == 4) { float f; memcpy(&f, s, 4); dv = f; }
            else if (dt.size == 8) { memcpy(&dv, s, 8); }
            else throw Error("unsupported float width");
        } else if (is_int) {
            uint64_t u = rd(s, dt.size);
            if (dt.is_signed && dt.size < 8 && (u >> (8 * dt.size - 1)) & 1) u |= ~uint64_t(0) << (8 * dt.size);
            iv = dt.is_signed ? int64_t(u) : int64_t(u);
            dv = double(iv);
        } else {
            throw Error("non-numeric element where a number was expected");
        }
        switch (kind) {
            case K_F32: static_cast<float*>(dst)[i] = is_int ? float(iv) : float(dv); break;
            case K_F64: static_cast<double*>(dst)[i] = is_int ? double(iv) : dv; break;
            case K_I32: static_cast<int32_t*>(dst)[i] = is_int ? int32_t(iv) : int32_t(dv); break;
            case K_I64: static_cast<int64_t*>(dst)[i] = is_int ? iv : int64_t(dv); break;
            default: throw Error("bad destination kind");
        }
    }
}

namespace {
template <typename T> int kind_of();
template <> int kind_of<float>() { return K_F32; }
template <> int kind_of<double>() { return K_F64; }
template <> int kind_of<int32_t>() { return K_I32; }
template <> int kind_of<int64_t>() { return K_I64; }

std::vector<std::string> split_strings(const Dtype& dt, const std::vector<uint8_t>& raw) {
    std::vector<std::string> out;
    if (dt.cls != DT_STRING) throw Error("value is not a fixed-length string");
    size_t w = size_t(dt.size);
    for (size_t i = 0; i + w <= raw.size(); i += w) {
        const char* c = reinterpret_cast<const char*>(raw.data() + i);
        size_t len = strnlen(c, w);
        while (len && c[len - 1] == ' ') --len;  // space-padded strings
        out.emplace_back(c, len);
    }
    return out;
}
}  // namespace

template <typename T>
std::vector<T> File::read(const std::string& path) {
    Object& o = resolve(path);
    auto raw = read_raw(path);
    size_t n = o.dt.size ? raw.size() / size_t(o.dt.size) : 0;
    std::vector<T> out(n);
    convert_elements(o.dt, raw.data(), n, kind_of<T>(), out.data());
    return out;
}
template std::vector<float> File::read<float>(const std::string&);
template std::vector<double> File::read<double>(const std::string&);
template std::vector<int32_t> File::read<int32_t>(const std::string&);
template std::vector<int64_t> File::read<int64_t>(const std::string&);

std::vector<std::string> File::read_strings(const std::string& path) {
    Object& o = resolve(path);
    return split_strings(o.dt, read_raw(path));
}

bool File::has_attr(const std::string& obj_path, const std::string& name) {
    Object& o = resolve(obj_path);
    for (auto& a : o.attrs)
        if (a.name == name) return true;
    return false;
}

const Attribute& File::attr(const std::string& obj_path, const std::string& name) {
    Object& o = resolve(obj_path);
    for (auto& a : o.attrs)
        if (a.name == name) return a;
    throw Error("attribute '" + name + "' not found on '" + obj_path + "'");
}

std::vector<std::string> File::attr_names(const std::string& obj_path) {
    std::vector<std::string> out;
    for (auto& a : resolve(obj_path).attrs) out.push_back(a.name);
    return out;
}

template <typename T>
std::vector<T> File::attr_values(const std::string& obj_path, const std::string& name) {
    const Attribute& a = attr(obj_path, name);
    size_t n = a.dt.size ? a.data.size() / size_t(a.dt.size) : 0;
    std::vector<T> out(n);
    convert_elements(a.dt, a.data.data(), n, kind_of<T>(), out.data());
    return out;
}
template std::vector<float> File::attr_values<float>(const std::string&, const std::string&);
template std::vector<double> File::attr_values<double>(const std::string&, const std::string&);
template std::vector<int32_t> File::attr_values<int32_t>(const std::string&, const std::string&);
template std::vector<int64_t> File::attr_values<int64_t>(const std::string&, const std::string&);

std::vector<std::string> File::attr_strings(const std::string& obj_path, const std::string& name) {
    const Attribute& a = attr(obj_path, name);
    return split_strings(a.dt, a.data);
}

}  // namespace h5lite
