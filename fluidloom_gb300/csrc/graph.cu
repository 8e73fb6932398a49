// graph.cu — execution graph: nodes with read/write field sets and AMR
// levels, hazard analysis, topological order, and a scheduler that runs the
// nodes on CUDA streams joined by events, replaying capturable stretches as
// cached CUDA graphs.
//
// Replaces the reference runtime: ExecutionNode (include/fluidloom/runtime/
// nodes/ExecutionNode.h:37-169), HazardAnalyzer (src/runtime/dependency/
// HazardAnalyzer.cpp:8-136: RAW, WAW, WAR and level barriers between every
// ordered pair of nodes, each hazard one edge), DependencyGraph (src/runtime/
// dependency/DependencyGraphBuilder.cpp:12-131: adjacency from the nodes'
// successor lists, Kahn's order with a FIFO ready queue, cycles rejected) and
// TopologicalScheduler (src/runtime/scheduler/TopologicalScheduler.cpp:16-71:
// nodes in topological order, each after its predecessors' completion).
// Where the reference chains one OpenCL event per node (TopologicalScheduler.cpp:
// 38-44 keeps only the last predecessor's), every predecessor on another
// stream is waited on here.
#include "common.cuh"

#include <chrono>
#include <cstring>
#include <deque>
#include <sstream>
#include <string>
#include <vector>

uint64_t fl_pool_launch_key(const fl_pool* P);
void fl_pool_advance_parity(fl_pool* P, int nsteps);

namespace {

constexpr int kMaxStreams = 8;

std::vector<std::string> split_fields(const char* s) {
    std::vector<std::string> out;
    if (!s) return out;
    std::string cur;
    for (const char* p = s;; ++p) {
        if (*p == ',' || *p == '\0') {
            size_t a = cur.find_first_not_of(" \t"), b = cur.find_last_not_of(" \t");
            if (a != std::string::npos) out.push_back(cur.substr(a, b - a + 1));
            cur.clear();
            if (*p == '\0') break;
        } else {
            cur.push_back(*p);
        }
    }
    return out;
}

bool contains(const std::vector<std::string>& v, const std::string& s) {
    for (const auto& x : v)
        if (x == s) return true;
    return false;
}

// Nodes that wait for the device on the host (a regrid reads counts back and
// reallocates) cannot be captured: they split the schedule into segments.
bool host_synchronizing(int type) { return type == FL_NODE_ADAPT_MESH; }

}  // namespace

struct fl_graph {
    fl_ctx* ctx = nullptr;
    struct Node {
        fl_node_desc d{};
        std::vector<std::string> reads, writes;
        std::vector<size_t> succ, pred;  // one entry per edge (hazards may repeat a pair)
        uint64_t count = 0;
        double total_ms = 0.0;
    };
    std::vector<Node> nodes;
    std::vector<fl_hazard> hazards;  // of the last fl_graph_analyze
    std::vector<size_t> order;
    size_t num_edges = 0;
    bool built = false;
    int profiling = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done;
    cudaEvent_t root = nullptr;
    struct Capture {
        std::vector<uint64_t> key;  // launch keys of the pools its steps touch, before it runs
        cudaGraphExec_t exec = nullptr;
        uint64_t kernels = 0;
    };
    struct Segment {
        size_t begin = 0, end = 0;  // positions in `order`
        std::deque<Capture> cache;  // most recent first (an odd step count alternates two keys)
    };
    std::vector<Segment> segs;
    std::string last_error;
};

namespace {

int graph_error(fl_graph* g, int code, const std::string& msg) {
    g->last_error = msg;
    if (g->ctx) return fl_set_error(g->ctx, code, msg);
    return code;
}

constexpr size_t kCapturesPerSegment = 4;

void drop_segments(fl_graph* g) {
    for (auto& s : g->segs)
        for (auto& c : s.cache) cudaGraphExecDestroy(c.exec);
    g->segs.clear();
}

int ensure_streams(fl_graph* g, size_t n) {
    while (g->streams.size() < n) {
        cudaStream_t s;
        FL_TRY_CUDA(g->ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "graph stream");
        g->streams.push_back(s);
    }
    while (g->done.size() < g->nodes.size()) {
        cudaEvent_t e;
        FL_TRY_CUDA(g->ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "graph event");
        g->done.push_back(e);
    }
    if (!g->root) FL_TRY_CUDA(g->ctx, cudaEventCreateWithFlags(&g->root, cudaEventDisableTiming), "graph event");
    return FL_OK;
}

// One node's work on stream s (the context stream is pointed at s meanwhile,
// so library calls made by the node land on it).
int run_node(fl_graph* g, fl_graph::Node& n, cudaStream_t s) {
    fl_ctx* ctx = g->ctx;
    cudaStream_t saved = ctx->stream;
    ctx->stream = s;
    int rc = FL_OK;
    switch (n.d.type) {
        case FL_NODE_KERNEL:
            if (n.d.fn) rc = n.d.fn(ctx, (void*)s, n.d.user);
            break;
        case FL_NODE_LBM_STEP:
            rc = n.d.pool ? fl_pool_step(ctx, n.d.pool, n.d.nsteps) : FL_E_INVALID_ARG;
            break;
        case FL_NODE_HOST:
            if (n.d.host_fn) {
                cudaError_t e = cudaLaunchHostFunc(s, (cudaHostFn_t)n.d.host_fn, n.d.user);
                if (e != cudaSuccess) rc = fl_check_cuda(ctx, e, "host node");
            }
            break;
        default:  // barriers, same-GPU halo exchange: ordering only
            break;
    }
    ctx->stream = saved;
    return rc;
}

// Emits positions [b, e) of the order (no host-synchronizing node among them)
// on the graph's streams, forked from and joined back into the context stream.
// A node continues the stream of its first predecessor that no earlier
// successor has continued; otherwise it takes the next stream.
int emit_segment(fl_graph* g, size_t b, size_t e, std::vector<cudaEvent_t>* timing) {
    fl_ctx* ctx = g->ctx;
    const size_t N = g->nodes.size();
    std::vector<int> stream_of(N, -1), pos(N, -1);
    std::vector<char> handed(N, 0);
    for (size_t k = b; k < e; ++k) pos[g->order[k]] = (int)k;
    int used = 0;
    for (size_t k = b; k < e; ++k) {
        const size_t i = g->order[k];
        for (size_t p : g->nodes[i].pred)
            if (pos[p] >= (int)b && !handed[p]) {
                stream_of[i] = stream_of[p];
                handed[p] = 1;
                break;
            }
        if (stream_of[i] < 0) stream_of[i] = used++ % kMaxStreams;
    }
    int rc = ensure_streams(g, (size_t)std::min(used, kMaxStreams));
    if (rc) return rc;
    const int ns = std::min(used, kMaxStreams);
    FL_TRY_CUDA(ctx, cudaEventRecord(g->root, ctx->stream), "graph fork");
    for (int s = 0; s < ns; ++s) FL_TRY_CUDA(ctx, cudaStreamWaitEvent(g->streams[s], g->root, 0), "graph fork");
    for (size_t k = b; k < e; ++k) {
        const size_t i = g->order[k];
        cudaStream_t st = g->streams[stream_of[i]];
        for (size_t p : g->nodes[i].pred)
            if (pos[p] >= (int)b && stream_of[p] != stream_of[i])
                FL_TRY_CUDA(ctx, cudaStreamWaitEvent(st, g->done[p], 0), "graph edge");
        if (timing) FL_TRY_CUDA(ctx, cudaEventRecord((*timing)[2 * i], st), "node timer");
        rc = run_node(g, g->nodes[i], st);
        if (rc) return rc;
        if (timing) FL_TRY_CUDA(ctx, cudaEventRecord((*timing)[2 * i + 1], st), "node timer");
        FL_TRY_CUDA(ctx, cudaEventRecord(g->done[i], st), "graph node");
    }
    for (int s = 0; s < ns; ++s) {
        cudaEvent_t last = nullptr;  // the last node emitted on stream s
        for (size_t k = b; k < e; ++k)
            if (stream_of[g->order[k]] == s) last = g->done[g->order[k]];
        if (last) FL_TRY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, last, 0), "graph join");
    }
    return FL_OK;
}

std::vector<uint64_t> segment_key(fl_graph* g, size_t b, size_t e) {
    std::vector<uint64_t> key;
    for (size_t k = b; k < e; ++k) {
        const auto& n = g->nodes[g->order[k]];
        if (n.d.type == FL_NODE_LBM_STEP && n.d.pool) {
            key.push_back((uint64_t)(uintptr_t)n.d.pool);
            key.push_back(fl_pool_launch_key(n.d.pool));
        }
    }
    return key;
}

int run_segment(fl_graph* g, fl_graph::Segment& sg, bool use_graphs, std::vector<cudaEvent_t>* timing) {
    fl_ctx* ctx = g->ctx;
    if (!use_graphs || timing) return emit_segment(g, sg.begin, sg.end, timing);
    std::vector<uint64_t> key = segment_key(g, sg.begin, sg.end);
    for (auto& c : sg.cache)
        if (c.key == key) {
            FL_TRY_CUDA(ctx, cudaGraphLaunch(c.exec, ctx->stream), "graph launch");
            ctx->launches += c.kernels;
            for (size_t k = sg.begin; k < sg.end; ++k) {
                auto& n = g->nodes[g->order[k]];
                if (n.d.type == FL_NODE_LBM_STEP && n.d.pool) fl_pool_advance_parity(n.d.pool, n.d.nsteps);
            }
            return FL_OK;
        }
    fl_graph::Capture c;
    c.key = key;
    const uint64_t c0 = ctx->launches;
    cudaGraph_t graph;
    FL_TRY_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    int rc = emit_segment(g, sg.begin, sg.end, nullptr);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
        if (ce == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
    }
    FL_TRY_CUDA(ctx, ce, "graph capture end");
    cudaError_t ie = cudaGraphInstantiate(&c.exec, graph, 0);
    cudaGraphDestroy(graph);
    FL_TRY_CUDA(ctx, ie, "graph instantiate");
    // the capture counted the launches it recorded and advanced the pools'
    // state as if they ran; the launch right below makes that true
    c.kernels = ctx->launches - c0;
    FL_TRY_CUDA(ctx, cudaGraphLaunch(c.exec, ctx->stream), "graph launch");
    sg.cache.push_front(c);
    if (sg.cache.size() > kCapturesPerSegment) {
        cudaGraphExecDestroy(sg.cache.back().exec);
        sg.cache.pop_back();
    }
    return FL_OK;
}

}  // namespace

extern "C" {

int fl_graph_create(fl_ctx* ctx, fl_graph** out) {
    if (!out) return FL_E_INVALID_ARG;
    *out = new fl_graph();
    (*out)->ctx = ctx;
    return FL_OK;
}

int fl_graph_destroy(fl_graph* g) {
    if (!g) return FL_E_INVALID_ARG;
    if (g->ctx) cudaStreamSynchronize(g->ctx->stream);
    drop_segments(g);
    for (auto s : g->streams) cudaStreamDestroy(s);
    for (auto e : g->done) cudaEventDestroy(e);
    if (g->root) cudaEventDestroy(g->root);
    delete g;
    return FL_OK;
}

const char* fl_graph_last_error(fl_graph* g) { return g ? g->last_error.c_str() : "null graph"; }

int fl_graph_add_node(fl_graph* g, const fl_node_desc* d, int64_t* id) {
    if (!g || !d) return FL_E_INVALID_ARG;
    if (d->type < FL_NODE_KERNEL || d->type > FL_NODE_HOST)
        return graph_error(g, FL_E_INVALID_ARG, "fl_graph_add_node: unknown node type");
    if ((d->type == FL_NODE_LBM_STEP || d->type == FL_NODE_ADAPT_MESH) && !d->pool)
        return graph_error(g, FL_E_INVALID_ARG, "fl_graph_add_node: step and adapt nodes need a pool");
    fl_graph::Node n;
    n.d = *d;
    n.d.name[sizeof(n.d.name) - 1] = '\0';
    n.reads = split_fields(d->reads);
    n.writes = split_fields(d->writes);
    n.d.reads = nullptr;  // the caller's strings are not kept
    n.d.writes = nullptr;
    g->nodes.push_back(std::move(n));
    g->built = false;
    drop_segments(g);
    if (id) *id = (int64_t)g->nodes.size() - 1;
    return FL_OK;
}

int fl_graph_add_edge(fl_graph* g, int64_t from, int64_t to) {
    if (!g || from < 0 || to < 0 || (size_t)from >= g->nodes.size() || (size_t)to >= g->nodes.size())
        return FL_E_INVALID_ARG;
    g->nodes[from].succ.push_back((size_t)to);
    g->nodes[to].pred.push_back((size_t)from);
    g->built = false;
    drop_segments(g);
    return FL_OK;
}

int fl_graph_analyze(fl_graph* g, fl_hazard* out, size_t cap, size_t* count) {
    if (!g) return FL_E_INVALID_ARG;
    std::vector<fl_hazard> hz;
    auto push = [&](size_t i, size_t j, const std::string& f, int type) {
        fl_hazard h{};
        h.from = i;
        h.to = j;
        h.type = type;
        std::strncpy(h.field, f.c_str(), sizeof(h.field) - 1);
        hz.push_back(h);
    };
    const auto& N = g->nodes;
    for (size_t i = 0; i < N.size(); ++i)  // RAW: a later node reads what this one writes
        for (size_t j = i + 1; j < N.size(); ++j)
            for (const auto& f : N[i].writes)
                if (contains(N[j].reads, f)) push(i, j, f, FL_HAZARD_RAW);
    for (size_t i = 0; i < N.size(); ++i)  // WAW
        for (size_t j = i + 1; j < N.size(); ++j)
            for (const auto& f : N[i].writes)
                if (contains(N[j].writes, f)) push(i, j, f, FL_HAZARD_WAW);
    for (size_t i = 0; i < N.size(); ++i)  // WAR: a later node writes what this one reads
        for (size_t j = i + 1; j < N.size(); ++j)
            for (const auto& f : N[i].reads)
                if (contains(N[j].writes, f)) push(i, j, f, FL_HAZARD_WAR);
    for (size_t i = 0; i < N.size(); ++i) {  // nodes on different AMR levels
        if (N[i].d.level < 0) continue;
        for (size_t j = i + 1; j < N.size(); ++j)
            if (N[j].d.level >= 0 && N[j].d.level != N[i].d.level) push(i, j, "", FL_HAZARD_LEVEL_BARRIER);
    }
    for (const auto& h : hz) {  // enforceHazards: one edge per hazard
        g->nodes[h.from].succ.push_back(h.to);
        g->nodes[h.to].pred.push_back(h.from);
    }
    g->hazards = hz;
    g->built = false;
    drop_segments(g);
    if (count) *count = hz.size();
    if (out)
        for (size_t k = 0; k < hz.size() && k < cap; ++k) out[k] = hz[k];
    return FL_OK;
}

int fl_graph_hazards(fl_graph* g, fl_hazard* out, size_t cap, size_t* n) {
    if (!g) return FL_E_INVALID_ARG;
    if (n) *n = g->hazards.size();
    if (out)
        for (size_t k = 0; k < g->hazards.size() && k < cap; ++k) out[k] = g->hazards[k];
    return FL_OK;
}

int fl_graph_build(fl_graph* g) {
    if (!g) return FL_E_INVALID_ARG;
    const size_t n = g->nodes.size();
    std::vector<size_t> indeg(n, 0);
    g->num_edges = 0;
    for (size_t i = 0; i < n; ++i)
        for (size_t s : g->nodes[i].succ) {
            ++indeg[s];
            ++g->num_edges;
        }
    std::deque<size_t> ready;
    for (size_t i = 0; i < n; ++i)
        if (!indeg[i]) ready.push_back(i);
    g->order.clear();
    while (!ready.empty()) {
        size_t i = ready.front();
        ready.pop_front();
        g->order.push_back(i);
        for (size_t s : g->nodes[i].succ)
            if (--indeg[s] == 0) ready.push_back(s);
    }
    drop_segments(g);
    if (g->order.size() != n) {
        g->built = false;
        return graph_error(g, FL_E_INVALID_ARG, "Dependency graph contains cycles");
    }
    // segments: maximal stretches of the order between host-synchronizing nodes
    size_t b = 0;
    for (size_t k = 0; k <= n; ++k) {
        if (k == n || host_synchronizing(g->nodes[g->order[k]].d.type)) {
            if (k > b) {
                fl_graph::Segment s;
                s.begin = b;
                s.end = k;
                g->segs.push_back(s);
            }
            b = k + 1;
        }
    }
    g->built = true;
    return FL_OK;
}

int fl_graph_num_edges(fl_graph* g, size_t* n) {
    if (!g || !n) return FL_E_INVALID_ARG;
    if (!g->built) return graph_error(g, FL_E_INVALID_ARG, "Graph not yet validated");
    *n = g->num_edges;
    return FL_OK;
}

int fl_graph_order(fl_graph* g, int64_t* ids, size_t cap, size_t* n) {
    if (!g) return FL_E_INVALID_ARG;
    if (!g->built) return graph_error(g, FL_E_INVALID_ARG, "Graph not yet validated");
    if (n) *n = g->order.size();
    if (ids)
        for (size_t k = 0; k < g->order.size() && k < cap; ++k) ids[k] = (int64_t)g->order[k];
    return FL_OK;
}

int fl_graph_set_profiling(fl_graph* g, int on) {
    if (!g) return FL_E_INVALID_ARG;
    g->profiling = on;
    return FL_OK;
}

int fl_graph_execute(fl_graph* g, int use_cuda_graphs) {
    if (!g || !g->ctx) return FL_E_INVALID_ARG;
    if (!g->built) return graph_error(g, FL_E_INVALID_ARG, "Graph not yet validated");
    fl_ctx* ctx = g->ctx;
    int rc = ensure_streams(g, 1);
    if (rc) return rc;
    std::vector<cudaEvent_t> timing;
    if (g->profiling) {
        timing.resize(2 * g->nodes.size());
        for (auto& e : timing) FL_TRY_CUDA(ctx, cudaEventCreate(&e), "node timer");
    }
    size_t si = 0;
    for (size_t k = 0; k < g->order.size();) {
        auto& n = g->nodes[g->order[k]];
        if (host_synchronizing(n.d.type)) {  // everything before it has joined the context stream
            auto t0 = std::chrono::steady_clock::now();
            fl_adapt_stats st{};
            rc = fl_pool_regrid(ctx, n.d.pool, &st);
            if (rc) return rc;
            if (g->profiling) {
                n.count++;
                n.total_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            }
            ++k;
            continue;
        }
        auto& sg = g->segs[si++];
        rc = run_segment(g, sg, use_cuda_graphs != 0, g->profiling ? &timing : nullptr);
        if (rc) return rc;
        k = sg.end;
    }
    if (g->profiling) {
        FL_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "profile sync");
        for (size_t i = 0; i < g->nodes.size(); ++i) {
            auto& n = g->nodes[i];
            if (host_synchronizing(n.d.type)) continue;
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, timing[2 * i], timing[2 * i + 1]) == cudaSuccess) {
                n.count++;
                n.total_ms += ms;
            }
        }
        for (auto e : timing) cudaEventDestroy(e);
    }
    return FL_OK;
}

int fl_graph_node_stats(fl_graph* g, int64_t id, uint64_t* count, double* total_ms) {
    if (!g || id < 0 || (size_t)id >= g->nodes.size()) return FL_E_INVALID_ARG;
    if (count) *count = g->nodes[id].count;
    if (total_ms) *total_ms = g->nodes[id].total_ms;
    return FL_OK;
}

int fl_graph_dot(fl_graph* g, char* buf, size_t cap, size_t* len) {
    if (!g) return FL_E_INVALID_ARG;
    static const char* kNames[] = {"KERNEL", "HALO_EXCHANGE", "BARRIER", "ADAPT_MESH", "LBM_STEP", "HOST"};
    std::ostringstream o;
    o << "digraph DependencyGraph {\n  rankdir=TB;\n";
    for (size_t i = 0; i < g->nodes.size(); ++i) {
        const auto& n = g->nodes[i];
        o << "  n" << i << " [label=\"" << n.d.name << "\\n" << kNames[n.d.type];
        if (n.d.level >= 0) o << " L" << n.d.level;
        o << "\"];\n";
        for (size_t s : n.succ) o << "  n" << i << " -> n" << s << ";\n";
    }
    o << "}\n";
    const std::string str = o.str();
    if (len) *len = str.size();
    if (buf && cap) {
        size_t m = std::min(cap - 1, str.size());
        std::memcpy(buf, str.data(), m);
        buf[m] = '\0';
    }
    return FL_OK;
}

}  // extern "C"
