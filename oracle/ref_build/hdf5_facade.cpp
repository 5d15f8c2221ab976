// Read-only implementation of the `hdf5.h` stand-in on top of h5lite.
// Test infrastructure: it exists so the reference engine can be compiled
// unmodified here as a CPU parity oracle.
#include "hdf5.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "h5lite.h"

namespace {

enum Kind { K_FILE, K_GROUP, K_DSET, K_SPACE, K_TYPE, K_ATTR, K_PLIST };

struct Handle {
    Kind kind;
    int refs = 1;
    std::shared_ptr<h5lite::File> file;
    std::string path;       // object path (file, group, dataset, attribute owner)
    std::string attr_name;  // for K_ATTR
    std::vector<hsize_t> dims;
    h5lite::Dtype dt;
};

std::map<hid_t, Handle> g_handles;
hid_t g_next = 1000;

hid_t make(Handle h) {
    hid_t id = g_next++;
    g_handles[id] = std::move(h);
    return id;
}

Handle* get(hid_t id) {
    auto it = g_handles.find(id);
    return it == g_handles.end() ? nullptr : &it->second;
}

herr_t release(hid_t id) {
    auto it = g_handles.find(id);
    if (it == g_handles.end()) return -1;
    if (--it->second.refs <= 0) g_handles.erase(it);
    return 0;
}

std::string join(const std::string& base, const char* name) {
    std::string n = name ? name : ".";
    if (!n.empty() && n[0] == '/') return n;
    if (n == ".") return base;
    return (base == "/" ? std::string("/") : base + "/") + n;
}

bool loc_path(hid_t loc, std::shared_ptr<h5lite::File>* f, std::string* path) {
    Handle* h = get(loc);
    if (!h || (h->kind != K_FILE && h->kind != K_GROUP && h->kind != K_DSET)) return false;
    *f = h->file;
    *path = h->path;
    return true;
}

int predef_kind(hid_t t, bool* is_uint) {
    *is_uint = false;
    if (t == H5T_NATIVE_FLOAT) return h5lite::K_F32;
    if (t == H5T_NATIVE_DOUBLE) return h5lite::K_F64;
    if (t == H5T_NATIVE_INT) return h5lite::K_I32;
    if (t == H5T_NATIVE_LONG) return h5lite::K_I64;
    if (t == H5T_NATIVE_UINT) { *is_uint = true; return h5lite::K_I64; }
    return -1;
}

herr_t convert_to(hid_t mem_type, const h5lite::Dtype& dt, const std::vector<uint8_t>& raw, void* buf) {
    size_t n = dt.size ? raw.size() / size_t(dt.size) : 0;
    bool is_uint;
    int kind = predef_kind(mem_type, &is_uint);
    try {
        if (kind >= 0) {
            if (is_uint) {
                std::vector<int64_t> tmp(n);
                h5lite::convert_elements(dt, raw.data(), n, kind, tmp.data());
                for (size_t i = 0; i < n; ++i) static_cast<uint32_t*>(buf)[i] = uint32_t(tmp[i]);
            } else {
                h5lite::convert_elements(dt, raw.data(), n, kind, buf);
            }
            return 0;
        }
        Handle* th = get(mem_type);
        if (th && th->kind == K_TYPE && dt.cls == h5lite::DT_STRING) {
            memcpy(buf, raw.data(), raw.size());  // same fixed-length string layout
            return 0;
        }
    } catch (const std::exception&) {
        return -1;
    }
    return -1;
}

}  // namespace

extern "C" {

hid_t H5Fopen(const char* name, unsigned flags, hid_t) {
    if (flags != H5F_ACC_RDONLY) return -1;
    try {
        Handle h{K_FILE};
        h.file = std::make_shared<h5lite::File>(name);
        h.path = "/";
        return make(std::move(h));
    } catch (const std::exception&) {
        return -1;
    }
}
hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return -1; }
herr_t H5Fclose(hid_t f) { return release(f); }
herr_t H5Fflush(hid_t, H5F_scope_t) { return 0; }

hid_t H5Gopen2(hid_t loc, const char* name, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    std::string p = join(base, name);
    try {
        if (!f->exists(p) || !f->is_group(p)) return -1;
    } catch (const std::exception&) {
        return -1;
    }
    Handle h{K_GROUP};
    h.file = f;
    h.path = p;
    return make(std::move(h));
}
hid_t H5Gcreate2(hid_t, const char*, hid_t, hid_t, hid_t) { return -1; }
herr_t H5Gclose(hid_t g) { return release(g); }

herr_t H5Gget_info_by_name(hid_t loc, const char* name, H5G_info_t* info, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    try {
        auto names = f->list(join(base, name));
        memset(info, 0, sizeof(*info));
        info->nlinks = names.size();
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

htri_t H5Lexists(hid_t loc, const char* name, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    return f->exists(join(base, name)) ? 1 : 0;
}
htri_t H5Oexists_by_name(hid_t loc, const char* name, hid_t lapl) { return H5Lexists(loc, name, lapl); }
herr_t H5Ldelete(hid_t, const char*, hid_t) { return -1; }

hssize_t H5Lget_name_by_idx(hid_t loc, const char* group_name, H5_index_t, H5_iter_order_t order, hsize_t n,
                            char* name, size_t size, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    try {
        auto names = f->list(join(base, group_name));  // sorted by name
        if (order == H5_ITER_DEC) std::reverse(names.begin(), names.end());
        if (n >= names.size()) return -1;
        const std::string& s = names[size_t(n)];
        if (name && size) {
            size_t k = std::min(size - 1, s.size());
            memcpy(name, s.data(), k);
            name[k] = 0;
        }
        return hssize_t(s.size());
    } catch (const std::exception&) {
        return -1;
    }
}

hid_t H5Dopen2(hid_t loc, const char* name, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    std::string p = join(base, name);
    try {
        if (!f->exists(p) || f->is_group(p)) return -1;
        Handle h{K_DSET};
        h.file = f;
        h.path = p;
        auto d = f->dims(p);
        h.dims.assign(d.begin(), d.end());
        h.dt = f->dtype(p);
        return make(std::move(h));
    } catch (const std::exception&) {
        return -1;
    }
}
hid_t H5Dcreate2(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return -1; }
herr_t H5Dclose(hid_t d) { return release(d); }

hid_t H5Dget_space(hid_t d) {
    Handle* h = get(d);
    if (!h || (h->kind != K_DSET && h->kind != K_ATTR)) return -1;
    Handle s{K_SPACE};
    s.dims = h->dims;
    return make(std::move(s));
}
hid_t H5Dget_type(hid_t d) {
    Handle* h = get(d);
    if (!h || (h->kind != K_DSET && h->kind != K_ATTR)) return -1;
    Handle t{K_TYPE};
    t.dt = h->dt;
    return make(std::move(t));
}

herr_t H5Dread(hid_t d, hid_t mem_type, hid_t, hid_t, hid_t, void* buf) {
    Handle* h = get(d);
    if (!h || h->kind != K_DSET) return -1;
    try {
        return convert_to(mem_type, h->dt, h->file->read_raw(h->path), buf);
    } catch (const std::exception&) {
        return -1;
    }
}
herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return -1; }
herr_t H5Dset_extent(hid_t, const hsize_t*) { return -1; }

hid_t H5Screate(H5S_class_t) { return make(Handle{K_SPACE}); }
hid_t H5Screate_simple(int rank, const hsize_t* dims, const hsize_t*) {
    Handle s{K_SPACE};
    s.dims.assign(dims, dims + rank);
    return make(std::move(s));
}
herr_t H5Sclose(hid_t s) { return release(s); }
int H5Sget_simple_extent_ndims(hid_t s) {
    Handle* h = get(s);
    return (h && h->kind == K_SPACE) ? int(h->dims.size()) : -1;
}
int H5Sget_simple_extent_dims(hid_t s, hsize_t* dims, hsize_t* maxdims) {
    Handle* h = get(s);
    if (!h || h->kind != K_SPACE) return -1;
    for (size_t i = 0; i < h->dims.size(); ++i) {
        if (dims) dims[i] = h->dims[i];
        if (maxdims) maxdims[i] = h->dims[i];
    }
    return int(h->dims.size());
}
herr_t H5Sselect_hyperslab(hid_t, H5S_seloper_t, const hsize_t*, const hsize_t*, const hsize_t*, const hsize_t*) {
    return 0;
}

htri_t H5Aexists_by_name(hid_t loc, const char* obj_name, const char* attr_name, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    try {
        return f->has_attr(join(base, obj_name), attr_name) ? 1 : 0;
    } catch (const std::exception&) {
        return -1;
    }
}

hid_t H5Aopen_by_name(hid_t loc, const char* obj_name, const char* attr_name, hid_t, hid_t) {
    std::shared_ptr<h5lite::File> f;
    std::string base;
    if (!loc_path(loc, &f, &base)) return -1;
    try {
        std::string p = join(base, obj_name);
        const auto& a = f->attr(p, attr_name);
        Handle h{K_ATTR};
        h.file = f;
        h.path = p;
        h.attr_name = attr_name;
        h.dims.assign(a.dims.begin(), a.dims.end());
        h.dt = a.dt;
        return make(std::move(h));
    } catch (const std::exception&) {
        return -1;
    }
}
hid_t H5Acreate_by_name(hid_t, const char*, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return -1; }

herr_t H5Aread(hid_t a, hid_t mem_type, void* buf) {
    Handle* h = get(a);
    if (!h || h->kind != K_ATTR) return -1;
    try {
        return convert_to(mem_type, h->dt, h->file->attr(h->path, h->attr_name).data, buf);
    } catch (const std::exception&) {
        return -1;
    }
}
herr_t H5Awrite(hid_t, hid_t, const void*) { return -1; }
herr_t H5Aclose(hid_t a) { return release(a); }
hid_t H5Aget_space(hid_t a) { return H5Dget_space(a); }
hid_t H5Aget_type(hid_t a) { return H5Dget_type(a); }

hid_t H5Tcopy(hid_t t) {
    Handle h{K_TYPE};
    if (t == H5T_C_S1) {
        h.dt.cls = h5lite::DT_STRING;
        h.dt.size = 1;
    } else if (Handle* o = get(t)) {
        h.dt = o->dt;
    }
    return make(std::move(h));
}
herr_t H5Tset_size(hid_t t, size_t size) {
    Handle* h = get(t);
    if (!h) return -1;
    h->dt.size = int(size);
    return 0;
}
herr_t H5Tset_strpad(hid_t, H5T_str_t) { return 0; }
size_t H5Tget_size(hid_t t) {
    Handle* h = get(t);
    return h ? size_t(h->dt.size) : 0;
}
htri_t H5Tis_variable_str(hid_t) { return 0; }
herr_t H5Tclose(hid_t t) { return release(t); }

hid_t H5Pcreate(hid_t) { return make(Handle{K_PLIST}); }
herr_t H5Pclose(hid_t p) { return release(p); }
herr_t H5Pset_chunk(hid_t, int, const hsize_t*) { return 0; }
herr_t H5Pset_shuffle(hid_t) { return 0; }
herr_t H5Pset_fletcher32(hid_t) { return 0; }
herr_t H5Pset_deflate(hid_t, unsigned) { return 0; }

int H5Iinc_ref(hid_t id) {
    Handle* h = get(id);
    if (!h) return -1;
    return ++h->refs;
}
herr_t H5Eset_auto(hid_t, void*, void*) { return 0; }

}  // extern "C"
