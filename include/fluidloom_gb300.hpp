// fluidloom_gb300.hpp — header-only C++17 layer over the C ABI that restores
// the reference's class and function names (fedres/fluidloom), so host code
// written against the reference's adaptation / hashmap / hilbert API keeps its
// shape.  Device buffers are CUDA device pointers where the reference passes
// cl_mem handles; errors throw fluidloom::FluidLoomError as the reference's
// FL_THROW does (include/fluidloom/common/FluidLoomError.h:13-81).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "fluidloom_gb300.h"

namespace fluidloom {

class FluidLoomError : public std::runtime_error {
public:
    FluidLoomError(int status, const std::string& msg)
        : std::runtime_error("[FluidLoomError] " + msg), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

inline void check(fl_ctx* ctx, int st, const char* what) {
    if (st != FL_OK && st != FL_E_BALANCE_NOT_CONVERGED)
        throw FluidLoomError(st, std::string(what) + ": " + (ctx ? fl_last_error(ctx) : fl_status_string(st)));
}

// Owns an fl_ctx (the reference passes a cl_context + cl_command_queue pair).
class Device {
public:
    explicit Device(int device = 0) { check(nullptr, fl_ctx_create(device, &ctx_), "fl_ctx_create"); }
    ~Device() { fl_ctx_destroy(ctx_); }
    Device(const Device&) = delete;
    Device& operator=(const Device&) = delete;
    fl_ctx* get() const { return ctx_; }
    void finish() { check(ctx_, fl_ctx_synchronize(ctx_), "finish"); }

private:
    fl_ctx* ctx_ = nullptr;
};

namespace hilbert {
// include/fluidloom/core/hilbert/HilbertCodec.h:29-68
using HilbertIndex = uint64_t;
static constexpr uint8_t COORDINATE_BITS = 21;
static constexpr HilbertIndex HILBERT_EMPTY = FL_EMPTY_KEY;
inline HilbertIndex encode(int32_t x, int32_t y, int32_t z, uint8_t level = 8) {
    return fl_hilbert_encode_host(x, y, z, level);
}
inline void decode(HilbertIndex h, uint8_t level, int32_t& x, int32_t& y, int32_t& z) {
    fl_hilbert_decode_host(h, level, &x, &y, &z);
}
inline HilbertIndex getParent(HilbertIndex h, uint8_t level) {
    if (level == 0) throw std::invalid_argument("Cannot get parent of level 0 cell");
    return fl_hilbert_get_parent(h, level);
}
inline HilbertIndex getChild(HilbertIndex h, uint8_t level, uint8_t quadrant) {
    if (level >= 21) throw std::invalid_argument("Cannot get child at max level");
    if (quadrant > 7) throw std::invalid_argument("Quadrant must be 0-7");
    return fl_hilbert_get_child(h, level, quadrant);
}
inline bool isValid(HilbertIndex h, uint8_t level) { return fl_hilbert_is_valid(h, level) != 0; }
}  // namespace hilbert

namespace adaptation {

// include/fluidloom/adaptation/AdaptationTypes.h:117-157 (key geometry added).
struct AdaptationConfig {
    uint8_t max_refinement_level = 8;
    uint8_t min_refinement_level = 0;
    uint32_t max_balance_iterations = 10;
    bool enforce_2_1_balance = true;
    int balance_mode = 0;  // 0: six face probes as the reference; 1: faces+edges+corners to a fixed point
    std::string default_averaging_rule = "arithmetic";
    double buffer_growth_factor = 1.5;
    int key_depth = 21;
    int anchor_level = 21;
    int32_t ext[3] = {1, 1, 1};
    int32_t periodic[3] = {0, 0, 0};
    bool input_balanced = false;  // the input has no FULL26 violation (fl_adapt_config.input_balanced)

    void validate() const {
        if (max_refinement_level > 21) throw std::invalid_argument("max_refinement_level cannot exceed 21");
        if (min_refinement_level > max_refinement_level)
            throw std::invalid_argument("min_refinement_level must be <= max_refinement_level");
    }
    fl_adapt_config c() const {
        fl_adapt_config k{};
        k.max_refinement_level = max_refinement_level;
        k.min_refinement_level = min_refinement_level;
        k.max_balance_iterations = max_balance_iterations;
        k.enforce_2_1_balance = enforce_2_1_balance;
        k.balance_mode = balance_mode;
        k.averaging_rule = default_averaging_rule == "volume_weighted" ? 1 : 0;
        k.buffer_growth_factor = buffer_growth_factor;
        k.key_depth = key_depth;
        k.anchor_level = anchor_level;
        for (int a = 0; a < 3; ++a) { k.ext[a] = ext[a]; k.periodic[a] = periodic[a]; }
        k.input_balanced = input_balanced ? 1 : 0;
        return k;
    }
};

using BalanceResult = fl_balance_result;

// Device leaf set with host helpers.
class Mesh {
public:
    Mesh(Device& dev, size_t capacity, bool with_case = false) : dev_(dev) {
        check(dev.get(), fl_mesh_alloc(dev.get(), capacity, with_case, &m_), "fl_mesh_alloc");
    }
    ~Mesh() { fl_mesh_free(dev_.get(), &m_); }
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;
    fl_mesh& raw() { return m_; }
    size_t size() const { return m_.num_cells; }
    void upload(const std::vector<int32_t>& x, const std::vector<int32_t>& y, const std::vector<int32_t>& z,
                const std::vector<uint8_t>& level, const std::vector<uint8_t>& state, const std::vector<int32_t>& flags,
                const std::vector<uint32_t>& material) {
        size_t n = x.size();
        if (n > m_.capacity) throw FluidLoomError(FL_E_CAPACITY, "mesh capacity");
        fl_ctx* c = dev_.get();
        check(c, fl_memcpy_h2d(c, m_.x, x.data(), n * 4), "upload");
        check(c, fl_memcpy_h2d(c, m_.y, y.data(), n * 4), "upload");
        check(c, fl_memcpy_h2d(c, m_.z, z.data(), n * 4), "upload");
        check(c, fl_memcpy_h2d(c, m_.level, level.data(), n), "upload");
        check(c, fl_memcpy_h2d(c, m_.state, state.data(), n), "upload");
        check(c, fl_memcpy_h2d(c, m_.flags, flags.data(), n * 4), "upload");
        check(c, fl_memcpy_h2d(c, m_.material, material.data(), n * 4), "upload");
        m_.num_cells = n;
    }
    template <typename T>
    std::vector<T> read(T* p) const {
        std::vector<T> v(m_.num_cells);
        if (!v.empty()) check(dev_.get(), fl_memcpy_d2h(dev_.get(), v.data(), p, v.size() * sizeof(T)), "read");
        return v;
    }

private:
    Device& dev_;
    fl_mesh m_{};
};

// AdaptationEngine::adapt (include/fluidloom/adaptation/AdaptationEngine.h:56-65).
class AdaptationEngine {
public:
    AdaptationEngine(Device& dev, const AdaptationConfig& cfg) : dev_(dev), cfg_(cfg) { cfg_.validate(); }
    fl_adapt_stats adapt(Mesh& mesh, float** fields = nullptr, uint32_t num_field_components = 0) {
        fl_adapt_stats st{};
        fl_adapt_config c = cfg_.c();
        check(dev_.get(), fl_adapt(dev_.get(), &mesh.raw(), &c, fields, num_field_components, &st), "adapt");
        return st;
    }

private:
    Device& dev_;
    AdaptationConfig cfg_;
};

// BalanceEnforcer::enforce (include/fluidloom/adaptation/BalanceEnforcer.h:48-53).
class BalanceEnforcer {
public:
    BalanceEnforcer(Device& dev, const AdaptationConfig& cfg) : dev_(dev), cfg_(cfg) {}
    BalanceResult enforce(Mesh& mesh) {
        BalanceResult r{};
        fl_adapt_config c = cfg_.c();
        check(dev_.get(), fl_balance_enforce(dev_.get(), &mesh.raw(), &c, &r), "enforce");
        return r;
    }

private:
    Device& dev_;
    AdaptationConfig cfg_;
};

// SplitEngine::split (include/fluidloom/adaptation/SplitEngine.h:51-59).
class SplitEngine {
public:
    SplitEngine(Device& dev, const AdaptationConfig& cfg) : dev_(dev), cfg_(cfg) {}
    size_t split(Mesh& parents, Mesh& children, const float* fields = nullptr, uint32_t C = 0,
                 float* child_fields = nullptr, uint32_t* parent_to_child = nullptr) {
        size_t nc = 0;
        fl_adapt_config c = cfg_.c();
        check(dev_.get(), fl_split(dev_.get(), &parents.raw(), &c, fields, C, &children.raw(), child_fields,
                                   parent_to_child, &nc), "split");
        return nc;
    }

private:
    Device& dev_;
    AdaptationConfig cfg_;
};

// MergeEngine::merge (include/fluidloom/adaptation/MergeEngine.h:51-59).
class MergeEngine {
public:
    MergeEngine(Device& dev, const AdaptationConfig& cfg) : dev_(dev), cfg_(cfg) {}
    size_t merge(Mesh& children, Mesh& parents, const float* fields = nullptr, uint32_t C = 0,
                 float* parent_fields = nullptr, uint32_t* merge_group_id = nullptr) {
        size_t np = 0;
        fl_adapt_config c = cfg_.c();
        check(dev_.get(), fl_merge(dev_.get(), &children.raw(), &c, fields, C, &parents.raw(), parent_fields,
                                   merge_group_id, &np), "merge");
        return np;
    }

private:
    Device& dev_;
    AdaptationConfig cfg_;
};

}  // namespace adaptation

namespace hashmap {

static constexpr uint64_t HASH_EMPTY_KEY = FL_EMPTY_KEY;
static constexpr uint32_t HASH_INVALID_VALUE = FL_INVALID;
static constexpr float MAX_LOAD_FACTOR = 0.6f;

// RadixSort::sortByKey (include/fluidloom/core/hashmap/RadixSort.h:33-35), device pointers.
class RadixSort {
public:
    explicit RadixSort(Device& dev) : dev_(dev) {}
    void sortByKey(uint64_t* keys, uint32_t* vals, size_t n, int begin_bit = 0, int end_bit = 64) {
        check(dev_.get(), fl_sort_pairs_u64_u32(dev_.get(), keys, vals, n, begin_bit, end_bit), "sortByKey");
    }
    // The sort's shape for the device context (fl_sort_set_config): 8- or 9-bit digits on
    // tiles of 256 or 512 threads; every shape gives the same order.
    void setShape(int digit_bits, int tile_threads) {
        check(dev_.get(), fl_sort_set_config(dev_.get(), digit_bits, tile_threads), "setShape");
    }

private:
    Device& dev_;
};

// HashTableManager (include/fluidloom/core/hashmap/HashTableManager.h:34-56), device pointers.
class HashTableManager {
public:
    explicit HashTableManager(Device& dev) : dev_(dev) {}
    ~HashTableManager() { release(); }
    static uint64_t computeCapacity(size_t n) { return fl_hash_compute_capacity(n); }
    void rebuild(const uint64_t* keys, const uint32_t* vals, size_t n) {
        uint64_t cap = computeCapacity(n);
        if (cap != capacity_) {
            release();
            check(dev_.get(), fl_device_alloc(dev_.get(), cap * 8, (void**)&tk_), "alloc");
            check(dev_.get(), fl_device_alloc(dev_.get(), cap * 4, (void**)&tv_), "alloc");
            capacity_ = cap;
        }
        check(dev_.get(), fl_hash_build(dev_.get(), tk_, tv_, capacity_, keys, vals, n), "rebuild");
        size_ = n;
    }
    void query(const uint64_t* q, uint32_t* out, size_t n) const {
        check(dev_.get(), fl_hash_query(dev_.get(), tk_, tv_, capacity_, q, out, n), "query");
    }
    uint64_t* getKeysDevicePtr() const { return tk_; }
    uint32_t* getValuesDevicePtr() const { return tv_; }
    uint64_t getCapacity() const { return capacity_; }

private:
    void release() {
        if (tk_) fl_device_free(dev_.get(), tk_);
        if (tv_) fl_device_free(dev_.get(), tv_);
        tk_ = nullptr;
        tv_ = nullptr;
        capacity_ = 0;
    }
    Device& dev_;
    uint64_t* tk_ = nullptr;
    uint32_t* tv_ = nullptr;
    uint64_t capacity_ = 0;
    size_t size_ = 0;
};

}  // namespace hashmap

namespace fields {

// SOAFieldManager (include/fluidloom/core/fields/SOAFieldManager.h:26-51) over one context:
// FieldHandle is the field id; device pointers are per component (component-major storage).
using FieldHandle = uint64_t;
class SOAFieldManager {
public:
    explicit SOAFieldManager(Device& dev) : dev_(dev) {}
    FieldHandle allocate(const fl_field_desc& desc, size_t num_cells) {
        FieldHandle h = 0;
        check(dev_.get(), fl_soa_allocate(dev_.get(), &desc, num_cells, &h), "SOAFieldManager::allocate");
        return h;
    }
    void deallocate(FieldHandle h) { check(dev_.get(), fl_soa_deallocate(dev_.get(), h), "SOAFieldManager::deallocate"); }
    void* getDevicePtr(FieldHandle h, uint16_t component = 0) const {
        void* p = nullptr;
        check(dev_.get(), fl_soa_device_ptr(dev_.get(), h, component, &p), "SOAFieldManager::getDevicePtr");
        return p;
    }
    size_t numCells(FieldHandle h) const {
        size_t n = 0;
        check(dev_.get(), fl_soa_info(dev_.get(), h, &n, nullptr, nullptr), "SOAFieldManager::numCells");
        return n;
    }
    uint64_t getVersion(FieldHandle h) const {
        uint64_t v = 0;
        check(dev_.get(), fl_soa_info(dev_.get(), h, nullptr, nullptr, &v), "SOAFieldManager::getVersion");
        return v;
    }

private:
    Device& dev_;
};

}  // namespace fields

namespace runtime {

// AdaptMeshNode (include/fluidloom/runtime/nodes/AdaptMeshNode.h:18-70): one regrid of a brick pool.
// LbmStepNode stands where the reference's generated lbm_* KernelNodes stand
// (include/fluidloom/runtime/nodes/KernelNode.h:27-73): one level-0 step.
class BrickPool {
public:
    BrickPool(Device& dev, const std::vector<fl_lbm_case>& cases) : dev_(dev), cases_(cases) {
        check(dev.get(), fl_pool_create(dev.get(), cases.data(), (int)cases.size(), &p_), "fl_pool_create");
    }
    ~BrickPool() { fl_pool_destroy(dev_.get(), p_); }
    BrickPool(const BrickPool&) = delete;
    BrickPool& operator=(const BrickPool&) = delete;
    fl_pool* get() const { return p_; }
    Device& device() const { return dev_; }
    fl_pool_info info() const {
        fl_pool_info i{};
        check(dev_.get(), fl_pool_info_get(dev_.get(), p_, &i), "info");
        return i;
    }
    // Solid voxels of one case at `level` (bit (z * Ny + y) * Nx + x, N = ext * 8 << level),
    // OR-ed with the case's sphere; an empty vector removes them (fl_pool_set_solid_mask).
    void setSolidMask(int32_t case_id, int32_t level, const std::vector<uint32_t>& bits) {
        check(dev_.get(),
              fl_pool_set_solid_mask(dev_.get(), p_, case_id, level, bits.empty() ? nullptr : bits.data(),
                                     bits.size()),
              "fl_pool_set_solid_mask");
    }
    // The populations as a 19-component field of the device's SOAFieldManager (a view of the pool's
    // current buffer, valid until the pool is stepped or regridded; fl_pool_populations_field).
    fields::FieldHandle populationsField(const std::string& name = "f") {
        fields::FieldHandle h = 0;
        check(dev_.get(), fl_pool_populations_field(dev_.get(), p_, name.c_str(), &h), "fl_pool_populations_field");
        return h;
    }
    // The case's mask level (-1: none) and words.
    int32_t solidMask(int32_t case_id, std::vector<uint32_t>* bits) const {
        int32_t level = -1;
        check(dev_.get(), fl_pool_get_solid_mask(dev_.get(), p_, case_id, &level, nullptr, 0), "fl_pool_get_solid_mask");
        if (level >= 0 && bits) {
            const fl_lbm_case& c = cases_.at(case_id);
            const uint64_t n = ((uint64_t)c.ext[0] * 8 << level) * ((uint64_t)c.ext[1] * 8 << level) *
                               ((uint64_t)c.ext[2] * 8 << level);
            bits->assign((size_t)((n + 31) / 32), 0u);
            check(dev_.get(), fl_pool_get_solid_mask(dev_.get(), p_, case_id, &level, bits->data(), bits->size()),
                  "fl_pool_get_solid_mask");
        }
        return level;
    }

private:
    Device& dev_;
    fl_pool* p_ = nullptr;
    std::vector<fl_lbm_case> cases_;
};

class LbmStepNode {
public:
    explicit LbmStepNode(BrickPool& pool, int steps = 1) : pool_(pool), steps_(steps) {}
    void execute() { check(pool_.device().get(), fl_pool_step(pool_.device().get(), pool_.get(), steps_), "step"); }

private:
    BrickPool& pool_;
    int steps_;
};

class AdaptMeshNode {
public:
    explicit AdaptMeshNode(BrickPool& pool) : pool_(pool) {}
    fl_adapt_stats execute() {
        fl_adapt_stats st{};
        check(pool_.device().get(), fl_pool_regrid(pool_.device().get(), pool_.get(), &st), "regrid");
        return st;
    }

private:
    BrickPool& pool_;
};

namespace dependency {

// The reference's DependencyGraph + HazardAnalyzer (include/fluidloom/runtime/dependency/
// DependencyGraph.h:21-107, HazardAnalyzer.h:20-86) over one fl_graph: nodes are added with
// their read/write field sets and level, analyzeNodes() enforces the hazards as edges,
// build() computes the topological order (throws on cycles, as the reference does).
class DependencyGraph {
public:
    enum class HazardType { RAW = FL_HAZARD_RAW, WAW = FL_HAZARD_WAW, WAR = FL_HAZARD_WAR,
                            LEVEL_BARRIER = FL_HAZARD_LEVEL_BARRIER };
    struct Hazard {
        size_t from_node_idx, to_node_idx;
        std::string field_name;
        HazardType type;
    };

    explicit DependencyGraph(fl_ctx* ctx = nullptr) : ctx_(ctx) {
        check(nullptr, fl_graph_create(ctx, &g_), "fl_graph_create");
    }
    ~DependencyGraph() { fl_graph_destroy(g_); }
    DependencyGraph(const DependencyGraph&) = delete;
    DependencyGraph& operator=(const DependencyGraph&) = delete;

    int64_t addNode(int type, const std::string& name, const std::string& reads, const std::string& writes,
                    int level = -1, fl_pool* pool = nullptr, int nsteps = 1, fl_node_fn fn = nullptr,
                    fl_host_fn host_fn = nullptr, void* user = nullptr) {
        fl_node_desc d{};
        d.type = type;
        name.copy(d.name, sizeof(d.name) - 1);
        d.level = level;
        d.reads = reads.c_str();
        d.writes = writes.c_str();
        d.pool = pool;
        d.nsteps = nsteps;
        d.fn = fn;
        d.host_fn = host_fn;
        d.user = user;
        int64_t id = -1;
        rc(fl_graph_add_node(g_, &d, &id), "addNode");
        return id;
    }
    void addEdge(int64_t from, int64_t to) { rc(fl_graph_add_edge(g_, from, to), "addEdge"); }

    std::vector<Hazard> analyzeNodes() {
        size_t n = 0;
        rc(fl_graph_analyze(g_, nullptr, 0, &n), "analyzeNodes");
        std::vector<fl_hazard> raw(n);
        rc(fl_graph_hazards(g_, raw.data(), n, &n), "hazards");
        std::vector<Hazard> out;
        for (const auto& h : raw) out.push_back({(size_t)h.from, (size_t)h.to, h.field, (HazardType)h.type});
        return out;
    }
    void build() { rc(fl_graph_build(g_), "build"); }
    std::vector<size_t> getTopologicalOrder() const {
        size_t n = 0;
        rc(fl_graph_order(g_, nullptr, 0, &n), "getTopologicalOrder");
        std::vector<int64_t> ids(n);
        rc(fl_graph_order(g_, ids.data(), n, &n), "getTopologicalOrder");
        return std::vector<size_t>(ids.begin(), ids.end());
    }
    size_t getNumEdges() const {
        size_t n = 0;
        rc(fl_graph_num_edges(g_, &n), "getNumEdges");
        return n;
    }
    std::string toDOT() const {
        size_t n = 0;
        rc(fl_graph_dot(g_, nullptr, 0, &n), "toDOT");
        std::string s(n + 1, '\0');
        rc(fl_graph_dot(g_, &s[0], n + 1, &n), "toDOT");
        s.resize(n);
        return s;
    }
    fl_graph* get() const { return g_; }
    fl_ctx* context() const { return ctx_; }

private:
    void rc(int st, const char* what) const {
        if (st != FL_OK) throw FluidLoomError(st, std::string(what) + ": " + fl_graph_last_error(g_));
    }
    fl_ctx* ctx_;
    fl_graph* g_ = nullptr;
};

}  // namespace dependency

namespace scheduler {

// TopologicalScheduler (include/fluidloom/runtime/scheduler/TopologicalScheduler.h:15-57):
// runs every node once in dependency order; execute() returns true on success like the
// reference and records the host-side schedule time.
class TopologicalScheduler {
public:
    explicit TopologicalScheduler(dependency::DependencyGraph& g, bool cuda_graphs = true)
        : g_(g), cuda_graphs_(cuda_graphs) {}
    bool execute() {
        int st = fl_graph_execute(g_.get(), cuda_graphs_ ? 1 : 0);
        if (st != FL_OK) throw FluidLoomError(st, std::string("execute: ") + fl_graph_last_error(g_.get()));
        return true;
    }

private:
    dependency::DependencyGraph& g_;
    bool cuda_graphs_;
};

}  // namespace scheduler
}  // namespace runtime
}  // namespace fluidloom
