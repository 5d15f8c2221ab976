// h5lite: a self-contained reader for the subset of the HDF5 file format that
// Upside `.up` configurations and force-field parameter files use.
//
// Upside stores its whole energy graph in HDF5 (`/input/potential/<node>`
// groups with `arguments` attributes and per-node datasets; the reference
// reads them through h5_support.h:85-260).  No HDF5 library is available on
// the build or GPU hosts, so this file implements the on-disk format directly:
//   - superblock versions 0 and 1, 8-byte offsets/lengths
//   - symbol-table groups (v1 B-tree type 0 + local heap + SNOD nodes)
//   - version-1 object headers with continuation blocks
//   - dataspace v1/v2, fixed-point / floating-point / fixed-string datatypes
//   - compact, contiguous and chunked layouts (layout message v1-v3)
//   - chunk filters: shuffle, deflate (own RFC 1951 decoder), fletcher32
//   - attribute messages v1-v3
// Anything outside that subset raises h5lite::Error with a clear message.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>
#include <map>
#include <memory>

namespace h5lite {

struct Error : public std::runtime_error {
    explicit Error(const std::string& s) : std::runtime_error(s) {}
};

enum DtypeClass { DT_INT = 0, DT_FLOAT = 1, DT_STRING = 3, DT_OTHER = 99 };

struct Dtype {
    int cls = DT_OTHER;
    int size = 0;           // bytes per element
    bool is_signed = false;
    bool big_endian = false;
    std::vector<uint8_t> raw;  // the datatype message as stored (Writer copies it verbatim)
};

struct Attribute {
    std::string name;
    Dtype dt;
    std::vector<uint64_t> dims;  // empty => scalar
    std::vector<uint8_t> data;
};

struct Object {
    uint64_t addr = 0;
    bool is_group = false;
    // group
    std::vector<std::pair<std::string, uint64_t>> links;
    // dataset
    Dtype dt;
    std::vector<uint64_t> dims;
    bool is_scalar = false;
    int layout_class = -1;      // 0 compact, 1 contiguous, 2 chunked
    uint64_t data_addr = 0, data_size = 0;
    std::vector<uint8_t> compact_data;
    std::vector<uint32_t> chunk_dims;  // includes trailing element-size dim
    std::vector<int> filters;          // filter ids in pipeline order
    std::vector<Attribute> attrs;
};

class File {
public:
    explicit File(const std::string& path);
    ~File();

    bool exists(const std::string& path);
    bool is_group(const std::string& path);
    std::vector<std::string> list(const std::string& group_path);
    std::vector<uint64_t> dims(const std::string& dset_path);
    Dtype dtype(const std::string& dset_path);

    // Read a numeric dataset converted to T (float, double, int32_t, int64_t).
    template <typename T> std::vector<T> read(const std::string& dset_path);
    // Read a fixed-length string dataset.
    std::vector<std::string> read_strings(const std::string& dset_path);
    // Raw element bytes (row-major, dims product * dtype.size).
    std::vector<uint8_t> read_raw(const std::string& dset_path);

    bool has_attr(const std::string& obj_path, const std::string& name);
    const Attribute& attr(const std::string& obj_path, const std::string& name);
    template <typename T> std::vector<T> attr_values(const std::string& obj_path, const std::string& name);
    std::vector<std::string> attr_strings(const std::string& obj_path, const std::string& name);
    std::vector<std::string> attr_names(const std::string& obj_path);

    const std::string& filename() const { return fname_; }

private:
    std::string fname_;
    std::vector<uint8_t> buf_;
    uint64_t base_ = 0;
    uint64_t root_addr_ = 0;
    std::map<uint64_t, std::unique_ptr<Object>> cache_;

    Object& load(uint64_t addr);
    Object& resolve(const std::string& path);
    void parse_header(Object& obj);
    void parse_message(Object& obj, int type, const uint8_t* p, size_t n);
    void read_group_btree(uint64_t btree_addr, uint64_t heap_data, std::vector<std::pair<std::string, uint64_t>>& out);
    void read_chunk_btree(const Object& obj, uint64_t addr, std::vector<uint8_t>& out);
    const uint8_t* at(uint64_t addr, size_t n) const;
};

// Writer for the same subset: symbol-table groups, version-1 object headers,
// contiguous datasets, attribute messages.  Build a tree in memory, then
// save() writes the whole file (to `<path>.tmp`, renamed over `path`, so a
// reader never sees a half-written file).  Groups hold at most 1024 links and
// an attribute at most 64 KiB (one object-header message).
class Writer {
public:
    struct Node {
        bool is_group = true;
        std::map<std::string, std::unique_ptr<Node>> children;
        std::vector<Attribute> attrs;
        Dtype dt;
        std::vector<uint64_t> dims;  // empty: scalar
        std::vector<uint8_t> data;
    };
    Writer();
    Node& group(const std::string& path);
    // dims empty => scalar; data holds product(dims) * dt.size bytes
    void dataset(const std::string& path, const Dtype& dt, const std::vector<uint64_t>& dims,
                 std::vector<uint8_t> data);
    // dims and data both empty => a null dataspace (no value)
    void attr(const std::string& path, const std::string& name, const Dtype& dt, const std::vector<uint64_t>& dims,
              std::vector<uint8_t> data);
    void remove(const std::string& path);
    void save(const std::string& filename) const;
    Node root;
};

// Datatype of a native little-endian number or fixed-length string.
Dtype dtype_int(int size, bool is_signed);
Dtype dtype_float(int size);
Dtype dtype_string(int size);

// Copy the object at src_path of `src` (group: recursively, with attributes)
// to dst_path of `dst`.  Datasets are written back contiguous and
// uncompressed; variable-length and reference data cannot be copied (Error).
// Links whose full path is in `skip` are left out.
void copy_tree(File& src, const std::string& src_path, Writer& dst, const std::string& dst_path,
               const std::vector<std::string>& skip = {});

// Element conversion helper shared with the Python binding.
void convert_elements(const Dtype& dt, const uint8_t* src, size_t n, int dst_kind, void* dst);
enum DstKind { K_F32 = 0, K_F64 = 1, K_I32 = 2, K_I64 = 3 };

// zlib-wrapped DEFLATE decoder (RFC 1950/1951).  Throws Error on corrupt input.
std::vector<uint8_t> inflate_zlib(const uint8_t* src, size_t n, size_t size_hint);

}  // namespace h5lite
