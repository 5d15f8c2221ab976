// h5lite writer: the output side of the HDF5 subset h5lite reads.
//
// Layout of a written file (all addresses 8 bytes, little-endian):
//   superblock version 0 (96 bytes, root symbol-table entry with its B-tree and
//   heap cached in the scratch pad); every group is a version-1 object header
//   with one symbol-table message pointing at a v1 B-tree of one leaf, one
//   symbol node (SNOD, room for 2 * LEAF_K links) and a local heap of link
//   names; every dataset is a version-1 object header with dataspace,
//   datatype and contiguous layout (version 3) messages and its data stored
//   after it; attributes are version-1 attribute messages.
// The upside driver writes its `/output` group this way (src/state_logger.h in
// the reference writes the same arrays through the HDF5 library).
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <set>

#include "h5lite.h"

namespace h5lite {

namespace {
constexpr uint64_t UNDEF = ~uint64_t(0);
constexpr int LEAF_K = 512;
constexpr int INTERNAL_K = 16;

struct Buf {
    std::vector<uint8_t> b;
    void put(const void* p, size_t n) {
        const uint8_t* q = static_cast<const uint8_t*>(p);
        b.insert(b.end(), q, q + n);
    }
    template <class T> void le(T v, int n = sizeof(T)) {
        for (int i = 0; i < n; ++i) b.push_back(uint8_t((uint64_t(v) >> (8 * i)) & 0xff));
    }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8() {
        while (b.size() % 8) b.push_back(0);
    }
    size_t size() const { return b.size(); }
};

std::vector<uint8_t> dtype_message(const Dtype& dt) {
    if (!dt.raw.empty()) return dt.raw;
    Buf m;
    if (dt.cls == DT_INT) {
        m.le<uint8_t>(0x10);
        m.le<uint8_t>(dt.is_signed ? 0x08 : 0x00);
        m.le<uint8_t>(0);
        m.le<uint8_t>(0);
        m.le<uint32_t>(uint32_t(dt.size));
        m.le<uint16_t>(0);
        m.le<uint16_t>(uint16_t(8 * dt.size));
    } else if (dt.cls == DT_FLOAT) {
        bool f4 = dt.size == 4;
        m.le<uint8_t>(0x11);
        m.le<uint8_t>(0x20);  // IEEE, mantissa normalised with implied bit
        m.le<uint8_t>(f4 ? 31 : 63);  // sign bit position
        m.le<uint8_t>(0);
        m.le<uint32_t>(uint32_t(dt.size));
        m.le<uint16_t>(0);                  // bit offset
        m.le<uint16_t>(f4 ? 32 : 64);       // precision
        m.le<uint8_t>(f4 ? 23 : 52);        // exponent location
        m.le<uint8_t>(f4 ? 8 : 11);         // exponent size
        m.le<uint8_t>(0);                   // mantissa location
        m.le<uint8_t>(f4 ? 23 : 52);        // mantissa size
        m.le<uint32_t>(f4 ? 127 : 1023);    // exponent bias
    } else if (dt.cls == DT_STRING) {
        m.le<uint8_t>(0x13);
        m.le<uint8_t>(0);  // null-terminated, ASCII
        m.le<uint8_t>(0);
        m.le<uint8_t>(0);
        m.le<uint32_t>(uint32_t(dt.size));
    } else {
        throw Error("h5lite writer: datatype without a stored description");
    }
    return m.b;
}

std::vector<uint8_t> dataspace_message(const std::vector<uint64_t>& dims) {
    Buf m;
    m.le<uint8_t>(1);
    m.le<uint8_t>(uint8_t(dims.size()));
    m.le<uint8_t>(0);
    m.le<uint8_t>(0);
    m.zeros(4);
    for (auto d : dims) m.le<uint64_t>(d);
    return m.b;
}

uint64_t n_elements(const std::vector<uint64_t>& dims) {
    uint64_t n = 1;
    for (auto d : dims) n *= d;
    return n;
}

void check_copyable(const Dtype& dt, const std::string& what) {
    int cls = dt.raw.empty() ? dt.cls : (dt.raw[0] & 15);
    if (cls == 7 || cls == 9) throw Error("cannot copy " + what + ": variable-length or reference data");
}

struct Emitter {
    Buf out;
    uint64_t root_tree = 0, root_heap = 0;

    uint64_t alloc(const std::vector<uint8_t>& blob) {
        out.pad8();
        uint64_t a = out.size();
        out.put(blob.data(), blob.size());
        return a;
    }

    uint64_t object(const Writer::Node& node, bool is_root) {
        std::vector<std::pair<int, std::vector<uint8_t>>> msgs;
        if (node.is_group) {
            if (node.children.size() > size_t(2 * LEAF_K))
                throw Error("h5lite writer: more than " + std::to_string(2 * LEAF_K) + " links in one group");
            std::vector<std::pair<std::string, uint64_t>> kids;
            for (auto& kv : node.children) kids.push_back({kv.first, object(*kv.second, false)});  // sorted by name
            Buf heap;
            heap.zeros(8);  // offset 0: the empty name
            std::vector<uint64_t> name_off;
            for (auto& k : kids) {
                name_off.push_back(heap.size());
                heap.put(k.first.c_str(), k.first.size() + 1);
                heap.pad8();
            }
            uint64_t heap_data = alloc(heap.b);
            Buf hh;
            hh.put("HEAP", 4);
            hh.zeros(4);
            hh.le<uint64_t>(heap.size());
            hh.le<uint64_t>(UNDEF);
            hh.le<uint64_t>(heap_data);
            uint64_t heap_addr = alloc(hh.b);
            Buf sn;
            sn.put("SNOD", 4);
            sn.le<uint8_t>(1);
            sn.le<uint8_t>(0);
            sn.le<uint16_t>(uint16_t(kids.size()));
            for (size_t i = 0; i < kids.size(); ++i) {
                sn.le<uint64_t>(name_off[i]);
                sn.le<uint64_t>(kids[i].second);
                sn.le<uint32_t>(0);  // no cached scratch
                sn.le<uint32_t>(0);
                sn.zeros(16);
            }
            sn.zeros(40 * (size_t(2 * LEAF_K) - kids.size()));
            uint64_t snod = alloc(sn.b);
            Buf tr;
            tr.put("TREE", 4);
            tr.le<uint8_t>(0);  // group node
            tr.le<uint8_t>(0);  // leaf
            tr.le<uint16_t>(kids.empty() ? 0 : 1);
            tr.le<uint64_t>(UNDEF);
            tr.le<uint64_t>(UNDEF);
            tr.le<uint64_t>(0);  // key 0: empty name
            tr.le<uint64_t>(snod);
            tr.le<uint64_t>(kids.empty() ? 0 : name_off.back());
            tr.zeros(size_t(2 * INTERNAL_K) * 16);
            uint64_t tree = alloc(tr.b);
            Buf st;
            st.le<uint64_t>(tree);
            st.le<uint64_t>(heap_addr);
            msgs.push_back({0x11, st.b});
            if (is_root) {
                root_tree = tree;
                root_heap = heap_addr;
            }
        } else {
            uint64_t nbytes = n_elements(node.dims) * uint64_t(node.dt.size);
            if (node.data.size() != nbytes)
                throw Error("h5lite writer: dataset holds " + std::to_string(node.data.size()) + " bytes, shape needs " +
                            std::to_string(nbytes));
            uint64_t data_addr = nbytes ? alloc(node.data) : UNDEF;
            msgs.push_back({0x01, dataspace_message(node.dims)});
            msgs.push_back({0x03, dtype_message(node.dt)});
            Buf lay;
            lay.le<uint8_t>(3);
            lay.le<uint8_t>(1);  // contiguous
            lay.le<uint64_t>(data_addr);
            lay.le<uint64_t>(nbytes);
            msgs.push_back({0x08, lay.b});
        }
        for (auto& a : node.attrs) {
            auto dt = dtype_message(a.dt);
            // no dims and no data: a null dataspace (version 2, type 2), as
            // PyTables stores an empty TITLE
            bool null_space = a.dims.empty() && a.data.empty();
            auto ds = null_space ? std::vector<uint8_t>{2, 0, 0, 2} : dataspace_message(a.dims);
            Buf m;
            m.le<uint8_t>(1);
            m.le<uint8_t>(0);
            m.le<uint16_t>(uint16_t(a.name.size() + 1));
            m.le<uint16_t>(uint16_t(dt.size()));
            m.le<uint16_t>(uint16_t(ds.size()));
            m.put(a.name.c_str(), a.name.size() + 1);
            m.pad8();
            m.put(dt.data(), dt.size());
            m.pad8();
            m.put(ds.data(), ds.size());
            m.pad8();
            m.put(a.data.data(), a.data.size());
            msgs.push_back({0x0C, m.b});
        }
        Buf body;
        for (auto& mm : msgs) {
            Buf padded;
            padded.put(mm.second.data(), mm.second.size());
            padded.pad8();
            if (padded.size() > 0xffff) throw Error("h5lite writer: object-header message above 64 KiB");
            body.le<uint16_t>(uint16_t(mm.first));
            body.le<uint16_t>(uint16_t(padded.size()));
            body.le<uint8_t>(0);
            body.zeros(3);
            body.put(padded.b.data(), padded.size());
        }
        if (msgs.empty()) {  // one NIL message
            body.le<uint16_t>(0);
            body.le<uint16_t>(8);
            body.zeros(4);
            body.zeros(8);
        }
        Buf hdr;
        hdr.le<uint8_t>(1);
        hdr.le<uint8_t>(0);
        hdr.le<uint16_t>(uint16_t(msgs.empty() ? 1 : msgs.size()));
        hdr.le<uint32_t>(1);
        hdr.le<uint32_t>(uint32_t(body.size()));
        hdr.zeros(4);
        hdr.put(body.b.data(), body.size());
        return alloc(hdr.b);
    }
};

std::vector<std::string> split_path(const std::string& path) {
    std::vector<std::string> parts;
    size_t i = 0;
    while (i < path.size()) {
        size_t j = path.find('/', i);
        if (j == std::string::npos) j = path.size();
        if (j > i) parts.push_back(path.substr(i, j - i));
        i = j + 1;
    }
    return parts;
}

std::string norm_path(const std::string& p) {
    std::string s;
    for (auto& part : split_path(p)) s += "/" + part;
    return s.empty() ? std::string("/") : s;
}

void copy_rec(File& src, const std::string& sp, Writer& dst, const std::string& dp, const std::set<std::string>& skip) {
    if (skip.count(sp)) return;
    if (src.is_group(sp)) {
        dst.group(dp);
        std::string base = sp == "/" ? "" : sp;
        std::string dbase = dp == "/" ? "" : dp;
        for (auto& child : src.list(sp)) copy_rec(src, base + "/" + child, dst, dbase + "/" + child, skip);
    } else {
        Dtype dt = src.dtype(sp);
        check_copyable(dt, "dataset '" + sp + "'");
        dst.dataset(dp, dt, src.dims(sp), src.read_raw(sp));
    }
    for (auto& an : src.attr_names(sp)) {
        const Attribute& a = src.attr(sp, an);
        check_copyable(a.dt, "attribute '" + an + "' of '" + sp + "'");
        dst.attr(dp, an, a.dt, a.dims, a.data);
    }
}
}  // namespace

Dtype dtype_int(int size, bool is_signed) {
    Dtype d;
    d.cls = DT_INT;
    d.size = size;
    d.is_signed = is_signed;
    return d;
}
Dtype dtype_float(int size) {
    Dtype d;
    d.cls = DT_FLOAT;
    d.size = size;
    d.is_signed = true;
    return d;
}
Dtype dtype_string(int size) {
    Dtype d;
    d.cls = DT_STRING;
    d.size = size;
    return d;
}

Writer::Writer() { root.is_group = true; }

Writer::Node& Writer::group(const std::string& path) {
    Node* cur = &root;
    for (auto& part : split_path(path)) {
        auto& slot = cur->children[part];
        if (!slot) slot.reset(new Node());
        if (!slot->is_group) throw Error("h5lite writer: '" + path + "' passes through a dataset");
        cur = slot.get();
    }
    return *cur;
}

void Writer::dataset(const std::string& path, const Dtype& dt, const std::vector<uint64_t>& dims,
                     std::vector<uint8_t> data) {
    auto parts = split_path(path);
    if (parts.empty()) throw Error("h5lite writer: empty dataset path");
    std::string name = parts.back();
    parts.pop_back();
    std::string parent;
    for (auto& p : parts) parent += "/" + p;
    Node& g = group(parent);
    std::unique_ptr<Node> n(new Node());
    n->is_group = false;
    n->dt = dt;
    n->dims = dims;
    if (data.size() != n_elements(dims) * uint64_t(dt.size))
        throw Error("h5lite writer: data for '" + path + "' does not match its shape");
    n->data = std::move(data);
    g.children[name] = std::move(n);
}

void Writer::attr(const std::string& path, const std::string& name, const Dtype& dt, const std::vector<uint64_t>& dims,
                  std::vector<uint8_t> data) {
    Node* cur = &root;
    for (auto& part : split_path(path)) {
        auto it = cur->children.find(part);
        if (it == cur->children.end()) throw Error("h5lite writer: no object '" + path + "'");
        cur = it->second.get();
    }
    if (!(dims.empty() && data.empty()) && data.size() != n_elements(dims) * uint64_t(dt.size))
        throw Error("h5lite writer: attribute '" + name + "' does not match its shape");
    for (auto& a : cur->attrs)
        if (a.name == name) {
            a.dt = dt;
            a.dims = dims;
            a.data = std::move(data);
            return;
        }
    Attribute a;
    a.name = name;
    a.dt = dt;
    a.dims = dims;
    a.data = std::move(data);
    cur->attrs.push_back(std::move(a));
}

void Writer::remove(const std::string& path) {
    auto parts = split_path(path);
    if (parts.empty()) return;
    Node* cur = &root;
    for (size_t i = 0; i + 1 < parts.size(); ++i) {
        auto it = cur->children.find(parts[i]);
        if (it == cur->children.end()) return;
        cur = it->second.get();
    }
    cur->children.erase(parts.back());
}

void Writer::save(const std::string& filename) const {
    Emitter em;
    em.out.zeros(96);
    uint64_t root_addr = em.object(root, true);
    uint64_t eof = em.out.size();
    Buf sb;
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    sb.put(sig, 8);
    const uint8_t ver[8] = {0, 0, 0, 0, 0, 8, 8, 0};
    sb.put(ver, 8);
    sb.le<uint16_t>(LEAF_K);
    sb.le<uint16_t>(INTERNAL_K);
    sb.le<uint32_t>(0);
    sb.le<uint64_t>(0);      // base address
    sb.le<uint64_t>(UNDEF);  // free-space info
    sb.le<uint64_t>(eof);
    sb.le<uint64_t>(UNDEF);  // driver info
    sb.le<uint64_t>(0);      // root link name offset
    sb.le<uint64_t>(root_addr);
    sb.le<uint32_t>(1);      // scratch pad caches the symbol table
    sb.le<uint32_t>(0);
    sb.le<uint64_t>(em.root_tree);
    sb.le<uint64_t>(em.root_heap);
    memcpy(em.out.b.data(), sb.b.data(), sb.size());
    std::string tmp = filename + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) throw Error("cannot open '" + tmp + "' for writing: " + strerror(errno));
    size_t w = fwrite(em.out.b.data(), 1, em.out.size(), f);
    int c = fclose(f);
    if (w != em.out.size() || c != 0) {
        std::remove(tmp.c_str());
        throw Error("write to '" + tmp + "' failed");
    }
    if (std::rename(tmp.c_str(), filename.c_str()) != 0) {
        std::remove(tmp.c_str());
        throw Error("cannot rename '" + tmp + "' to '" + filename + "': " + strerror(errno));
    }
}

void copy_tree(File& src, const std::string& src_path, Writer& dst, const std::string& dst_path,
               const std::vector<std::string>& skip) {
    std::set<std::string> skip_norm;
    for (auto& s : skip) skip_norm.insert(norm_path(s));
    copy_rec(src, norm_path(src_path), dst, norm_path(dst_path), skip_norm);
}

}  // namespace h5lite
