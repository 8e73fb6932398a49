// fields.cu — field descriptors, the process-wide field registry and the
// per-context structure-of-arrays field manager.
//
// Replaces FieldDescriptor (include/fluidloom/core/fields/FieldDescriptor.h:40-83,
// validation src/core/fields/FieldDescriptor.cpp:8-43), FieldRegistry
// (src/core/registry/FieldRegistry.cpp:7-66) and SOAFieldManager
// (src/core/fields/SOAFieldManager.cpp:17-202).  Ids are FNV-1a 64 of the name
// (include/fluidloom/common/Hash.h:13-22, bytes taken unsigned so the id does
// not depend on the platform's char signedness).  Deviation: components are
// laid out component-major with a 128-byte aligned pitch (the reference's
// component pointers are base + comp * bytes_per_cell, which overlap when a
// field has more than one component, SOAFieldManager.cpp:50-54).
#include "common.cuh"

#include <cstring>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <unordered_map>

namespace {

uint64_t fnv1a_64(const char* s) {
    uint64_t h = 14695981039346656037ull;
    for (const unsigned char* p = (const unsigned char*)s; *p; ++p) {
        h ^= (uint64_t)*p;
        h *= 1099511628211ull;
    }
    return h;
}

size_t type_size(int32_t t) {
    switch (t) {
        case 0: return 4;  // FLOAT32
        case 1: return 8;  // FLOAT64
        case 2: return 4;  // INT32
        case 3: return 8;  // INT64
        case 4: return 1;  // UINT8
        default: return 0;
    }
}

struct Registry {
    std::shared_mutex mu;
    std::unordered_map<std::string, fl_field_desc> by_name;
    std::unordered_map<uint64_t, fl_field_desc> by_id;
};

Registry& registry() {
    static Registry r;
    return r;
}

struct FieldState {
    fl_field_desc desc;
    size_t num_cells = 0;
    size_t pitch = 0;  // bytes between components
    void* base = nullptr;
    uint64_t version = 1;
    bool external = false;  // storage owned elsewhere (a pool's populations): never freed or resized here
};

struct SoaManager {
    std::mutex mu;
    std::unordered_map<uint64_t, FieldState> fields;
};

size_t pitch_of(const fl_field_desc& d, size_t n) {
    size_t b = type_size(d.type) * n;
    return (b + 127) & ~(size_t)127;
}

int validate(const fl_field_desc* d, fl_ctx* ctx) {
    size_t len = strnlen(d->name, sizeof(d->name));
    if (len == 0 || len > 64) return fl_set_error(ctx, FL_E_INVALID_ARG, "Field name must be 1-64 characters");
    if (d->num_components == 0 || d->num_components > 32)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "num_components must be in [1,32]");
    if (d->halo_depth > 2) return fl_set_error(ctx, FL_E_INVALID_ARG, "halo_depth must be 0, 1, or 2");
    if (type_size(d->type) == 0) return fl_set_error(ctx, FL_E_INVALID_ARG, "unknown field type");
    return FL_OK;
}

}  // namespace

void fl_soa_release_all(fl_ctx* ctx) {
    if (!ctx || !ctx->soa) return;
    SoaManager* m = (SoaManager*)ctx->soa;
    for (auto& kv : m->fields)
        if (kv.second.base && !kv.second.external) cudaFree(kv.second.base);
    delete m;
    ctx->soa = nullptr;
}

extern "C" {

uint64_t fl_fnv1a_64(const char* s) { return s ? fnv1a_64(s) : 0; }

size_t fl_field_bytes_per_cell(const fl_field_desc* d) {
    return d ? type_size(d->type) * (size_t)d->num_components : 0;
}

int fl_field_make(const char* name, int32_t type, uint16_t components, uint8_t halo_depth, uint8_t avg_rule,
                  uint8_t solid_scheme, fl_field_desc* out) {
    if (!name || !out) return FL_E_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    size_t len = strnlen(name, 80);
    if (len >= sizeof(out->name)) return FL_E_INVALID_ARG;
    std::memcpy(out->name, name, len);
    out->type = type;
    out->num_components = components;
    out->halo_depth = halo_depth;
    out->avg_rule = avg_rule;
    out->solid_scheme = solid_scheme;
    int rc = validate(out, nullptr);
    if (rc) return rc;
    out->id = fnv1a_64(out->name);
    return FL_OK;
}

int fl_field_register(const fl_field_desc* d) {
    if (!d || validate(d, nullptr)) return FL_E_INVALID_ARG;
    Registry& r = registry();
    std::unique_lock<std::shared_mutex> lock(r.mu);
    std::string name(d->name);
    if (r.by_name.count(name)) return FL_E_CAPACITY;  // a field of that name exists (registerField returns false)
    fl_field_desc c = *d;
    c.id = fnv1a_64(c.name);
    r.by_name[name] = c;
    r.by_id[c.id] = c;
    return FL_OK;
}

int fl_field_lookup_name(const char* name, fl_field_desc* out) {
    if (!name || !out) return FL_E_INVALID_ARG;
    Registry& r = registry();
    std::shared_lock<std::shared_mutex> lock(r.mu);
    auto it = r.by_name.find(name);
    if (it == r.by_name.end()) return FL_E_INVALID_ARG;
    *out = it->second;
    return FL_OK;
}

int fl_field_lookup_id(uint64_t id, fl_field_desc* out) {
    if (!out) return FL_E_INVALID_ARG;
    Registry& r = registry();
    std::shared_lock<std::shared_mutex> lock(r.mu);
    auto it = r.by_id.find(id);
    if (it == r.by_id.end()) return FL_E_INVALID_ARG;
    *out = it->second;
    return FL_OK;
}

size_t fl_field_registry_count(void) {
    Registry& r = registry();
    std::shared_lock<std::shared_mutex> lock(r.mu);
    return r.by_name.size();
}

void fl_field_registry_clear(void) {
    Registry& r = registry();
    std::unique_lock<std::shared_mutex> lock(r.mu);
    r.by_name.clear();
    r.by_id.clear();
}

int fl_soa_allocate(fl_ctx* ctx, const fl_field_desc* d, size_t num_cells, uint64_t* handle) {
    if (!ctx || !d || !handle) return FL_E_INVALID_ARG;
    int rc = validate(d, ctx);
    if (rc) return rc;
    if (!ctx->soa) ctx->soa = new SoaManager();
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    uint64_t id = fnv1a_64(d->name);
    if (m->fields.count(id)) return fl_set_error(ctx, FL_E_INVALID_ARG, "Field already allocated");
    FieldState st;
    st.desc = *d;
    st.desc.id = id;
    st.num_cells = num_cells;
    st.pitch = pitch_of(*d, num_cells);
    size_t bytes = st.pitch * d->num_components;
    if (bytes) FL_TRY_CUDA(ctx, fl_dev_malloc(ctx, (void**)&st.base, bytes), "fl_soa_allocate");
    if (bytes) FL_TRY_CUDA(ctx, cudaMemsetAsync(st.base, 0, bytes, ctx->stream), "fl_soa_allocate zero");
    m->fields[id] = st;
    *handle = id;
    return FL_OK;
}

int fl_soa_resize(fl_ctx* ctx, uint64_t handle, size_t new_num_cells) {
    if (!ctx || !ctx->soa) return FL_E_INVALID_ARG;
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    auto it = m->fields.find(handle);
    if (it == m->fields.end()) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_soa_resize: unknown field");
    FieldState& st = it->second;
    if (st.external) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_soa_resize: the field's storage belongs to a pool");
    if (new_num_cells == st.num_cells) return FL_OK;
    size_t np = pitch_of(st.desc, new_num_cells);
    void* nb = nullptr;
    size_t bytes = np * st.desc.num_components;
    if (bytes) {
        FL_TRY_CUDA(ctx, fl_dev_malloc(ctx, (void**)&nb, bytes), "fl_soa_resize");
        FL_TRY_CUDA(ctx, cudaMemsetAsync(nb, 0, bytes, ctx->stream), "fl_soa_resize zero");
    }
    size_t keep = type_size(st.desc.type) * (new_num_cells < st.num_cells ? new_num_cells : st.num_cells);
    for (uint16_t c = 0; c < st.desc.num_components && keep; ++c)
        FL_TRY_CUDA(ctx, cudaMemcpyAsync((char*)nb + c * np, (char*)st.base + c * st.pitch, keep,
                                         cudaMemcpyDeviceToDevice, ctx->stream), "fl_soa_resize copy");
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_soa_resize");
    if (st.base) cudaFree(st.base);
    st.base = nb;
    st.pitch = np;
    st.num_cells = new_num_cells;
    st.version++;
    return FL_OK;
}

int fl_soa_deallocate(fl_ctx* ctx, uint64_t handle) {
    if (!ctx || !ctx->soa) return FL_E_INVALID_ARG;
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    auto it = m->fields.find(handle);
    if (it == m->fields.end()) return FL_OK;  // the reference only warns
    FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "fl_soa_deallocate");
    if (it->second.base && !it->second.external) cudaFree(it->second.base);
    m->fields.erase(it);
    return FL_OK;
}

int fl_soa_device_ptr(fl_ctx* ctx, uint64_t handle, uint16_t component, void** out) {
    if (!ctx || !ctx->soa || !out) return FL_E_INVALID_ARG;
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    auto it = m->fields.find(handle);
    if (it == m->fields.end()) return fl_set_error(ctx, FL_E_INVALID_ARG, "fl_soa_device_ptr: unknown field");
    if (component >= it->second.desc.num_components)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "Component index out of range");
    *out = (char*)it->second.base + component * it->second.pitch;
    return FL_OK;
}

int fl_soa_info(fl_ctx* ctx, uint64_t handle, size_t* num_cells, size_t* pitch_bytes, uint64_t* version) {
    if (!ctx || !ctx->soa) return FL_E_INVALID_ARG;
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    auto it = m->fields.find(handle);
    if (it == m->fields.end()) return FL_E_INVALID_ARG;
    if (num_cells) *num_cells = it->second.num_cells;
    if (pitch_bytes) *pitch_bytes = it->second.pitch;
    if (version) *version = it->second.version;
    return FL_OK;
}

size_t fl_soa_total_bytes(fl_ctx* ctx) {
    if (!ctx || !ctx->soa) return 0;
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    size_t t = 0;
    for (auto& kv : m->fields) t += kv.second.pitch * kv.second.desc.num_components;
    return t;
}

}  // extern "C"

// A field of the context's manager over storage owned elsewhere (component c at
// base + c * pitch bytes, num_cells cells); binding the same name again points
// it at the new storage and bumps its version when anything changed.
int fl_soa_bind_external(fl_ctx* ctx, const fl_field_desc* d, size_t num_cells, size_t pitch, void* base,
                         uint64_t* handle) {
    if (!ctx || !d || !handle) return FL_E_INVALID_ARG;
    int rc = validate(d, ctx);
    if (rc) return rc;
    if (!ctx->soa) ctx->soa = new SoaManager();
    SoaManager* m = (SoaManager*)ctx->soa;
    std::lock_guard<std::mutex> lock(m->mu);
    const uint64_t id = fnv1a_64(d->name);
    auto it = m->fields.find(id);
    if (it != m->fields.end() && !it->second.external)
        return fl_set_error(ctx, FL_E_INVALID_ARG, "a field of that name is allocated by the manager");
    FieldState& st = m->fields[id];
    const bool changed = st.base != base || st.pitch != pitch || st.num_cells != num_cells;
    st.desc = *d;
    st.desc.id = id;
    st.num_cells = num_cells;
    st.pitch = pitch;
    st.base = base;
    st.external = true;
    if (changed && it != m->fields.end()) st.version++;
    *handle = id;
    return FL_OK;
}
