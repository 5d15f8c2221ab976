// Plain C entry points over h5lite so Python (ctypes) can read `.up` files and
// parameter libraries without an HDF5 library.
#include "h5lite.h"

#include <cstring>
#include <string>

using h5lite::File;

namespace {
thread_local std::string g_err;

int put_list(const std::vector<std::string>& names, char* out, int outlen) {
    std::string s;
    for (auto& n : names) { s += n; s += '\n'; }
    if (int(s.size()) + 1 > outlen) return int(s.size()) + 1;
    memcpy(out, s.c_str(), s.size() + 1);
    return 0;
}

void put_shape(const h5lite::Dtype& dt, const std::vector<uint64_t>& dims, int64_t* out_dims, int maxrank,
               int* info) {
    for (size_t i = 0; i < dims.size() && int(i) < maxrank; ++i) out_dims[i] = int64_t(dims[i]);
    info[0] = dt.cls;
    info[1] = dt.size;
    info[2] = dt.is_signed;
    info[3] = dt.big_endian;
}
}  // namespace

#define GUARD(expr)                                   \
    try {                                             \
        expr;                                         \
    } catch (const std::exception& e) {               \
        g_err = e.what();                             \
        return -1;                                    \
    }

extern "C" {

const char* h5l_last_error() { return g_err.c_str(); }

void* h5l_open(const char* path) {
    try {
        return new File(path);
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void h5l_close(void* f) { delete static_cast<File*>(f); }

// -1 missing, 0 dataset, 1 group
int h5l_kind(void* f, const char* path) {
    File* F = static_cast<File*>(f);
    GUARD(if (!F->exists(path)) return -1; return F->is_group(path) ? 1 : 0;)
}

int h5l_list(void* f, const char* path, char* out, int outlen) {
    GUARD(return put_list(static_cast<File*>(f)->list(path), out, outlen);)
}

// returns rank; info = {class, size, signed, big_endian}
int h5l_shape(void* f, const char* path, int64_t* dims, int maxrank, int* info) {
    File* F = static_cast<File*>(f);
    GUARD(auto d = F->dims(path); put_shape(F->dtype(path), d, dims, maxrank, info); return int(d.size());)
}

int h5l_read_raw(void* f, const char* path, void* out, int64_t nbytes) {
    GUARD(auto raw = static_cast<File*>(f)->read_raw(path);
          if (int64_t(raw.size()) != nbytes) { g_err = "size mismatch"; return -1; }
          memcpy(out, raw.data(), raw.size()); return 0;)
}

int h5l_attr_names(void* f, const char* path, char* out, int outlen) {
    GUARD(return put_list(static_cast<File*>(f)->attr_names(path), out, outlen);)
}

int h5l_attr_shape(void* f, const char* path, const char* name, int64_t* dims, int maxrank, int* info) {
    GUARD(auto& a = static_cast<File*>(f)->attr(path, name); put_shape(a.dt, a.dims, dims, maxrank, info);
          info[4] = int(a.data.size()); return int(a.dims.size());)
}

// Rewrite `src` as `dst` with the h5lite writer, leaving out the
// '\n'-separated paths in `skip` (may be empty or NULL).
int h5l_copy_file(const char* src, const char* dst, const char* skip) {
    GUARD(File f(src); h5lite::Writer w; std::vector<std::string> sk; std::string s = skip ? skip : "";
          size_t i = 0; while (i < s.size()) { size_t j = s.find('\n', i); if (j == std::string::npos) j = s.size();
                                               if (j > i) sk.push_back(s.substr(i, j - i)); i = j + 1; }
          h5lite::copy_tree(f, "/", w, "/", sk); w.save(dst); return 0;)
}

int h5l_attr_read_raw(void* f, const char* path, const char* name, void* out, int64_t nbytes) {
    GUARD(auto& a = static_cast<File*>(f)->attr(path, name);
          if (int64_t(a.data.size()) != nbytes) { g_err = "size mismatch"; return -1; }
          memcpy(out, a.data.data(), a.data.size()); return 0;)
}
}
