// C++ host-side parity checks through include/fluidloom_gb300.hpp, in the
// shape of the reference's gtest cases (tests/unit/adaptation/*Test.cpp,
// tests/unit/hilbert/test_hilbert_codec.cpp).  Built and run by
// tests/test_gpu_cpp.py; prints "ALL PASSED" and exits 0 on success.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fluidloom_gb300.hpp"

using namespace fluidloom;
using namespace fluidloom::adaptation;

static int failures = 0;
#define EXPECT_EQ(a, b)                                                                          \
    do {                                                                                         \
        auto _a = (a);                                                                           \
        auto _b = (b);                                                                           \
        if (!(_a == _b)) {                                                                       \
            std::printf("%s:%d EXPECT_EQ(%s, %s) failed\n", __FILE__, __LINE__, #a, #b);          \
            ++failures;                                                                          \
        }                                                                                        \
    } while (0)
#define EXPECT_TRUE(a) EXPECT_EQ(!!(a), true)

int main() {
    // test_hilbert_codec.cpp:33-58, 108-125
    EXPECT_EQ(hilbert::encode(0, 0, 0, 1), 0ull);
    std::vector<int> seen(8, 0);
    for (int z = 0; z < 2; ++z)
        for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x) seen[hilbert::encode(x, y, z, 1)]++;
    for (int i = 0; i < 8; ++i) EXPECT_EQ(seen[i], 1);
    for (int lv = 1; lv <= 21; ++lv) {
        int32_t x = (12345 * lv) & ((1 << lv) - 1), y = (777 * lv) & ((1 << lv) - 1), z = (31 * lv) & ((1 << lv) - 1);
        int32_t a, b, c;
        hilbert::decode(hilbert::encode(x, y, z, lv), lv, a, b, c);
        EXPECT_EQ(a, x); EXPECT_EQ(b, y); EXPECT_EQ(c, z);
        EXPECT_TRUE(hilbert::isValid(hilbert::encode(x, y, z, lv), lv));
    }
    Device dev(0);
    AdaptationConfig cfg;
    cfg.max_refinement_level = 8;
    // SplitEngineTest.cpp:35-63
    {
        Mesh parents(dev, 1), children(dev, 8);
        parents.upload({0}, {0}, {0}, {0}, {0}, {1}, {0});
        SplitEngine se(dev, cfg);
        EXPECT_EQ(se.split(parents, children), (size_t)8);
        for (uint8_t l : children.read(children.raw().level)) EXPECT_EQ((int)l, 1);
    }
    // MergeEngineTest.cpp:35-71
    {
        Mesh kids(dev, 8), parents(dev, 1);
        std::vector<int32_t> x(8), y(8), z(8);
        for (int i = 0; i < 8; ++i) { x[i] = i & 1; y[i] = (i >> 1) & 1; z[i] = (i >> 2) & 1; }
        kids.upload(x, y, z, std::vector<uint8_t>(8, 1), std::vector<uint8_t>(8, 0), std::vector<int32_t>(8, -1),
                    std::vector<uint32_t>(8, 0));
        MergeEngine me(dev, cfg);
        EXPECT_EQ(me.merge(kids, parents), (size_t)1);
        EXPECT_EQ((int)parents.read(parents.raw().level)[0], 0);
        EXPECT_EQ(parents.read(parents.raw().x)[0], 0);
    }
    // BalanceEnforcerTest.cpp:37-93 (8-level anchors: x = {0, 128} -> native {0, 4})
    {
        Mesh m(dev, 2);
        m.upload({0, 4}, {0, 0}, {0, 0}, {1, 3}, {0, 0}, {0, 0}, {0, 0});
        AdaptationConfig c8 = cfg;
        c8.anchor_level = 8;
        BalanceEnforcer be(dev, c8);
        BalanceResult r = be.enforce(m);
        EXPECT_TRUE(r.converged);
        EXPECT_TRUE(r.total_violations_detected > 0);
        EXPECT_TRUE(r.total_cells_marked_for_balance > 0);
        auto f = m.read(m.raw().flags);
        EXPECT_EQ(f[0], 1);
        EXPECT_EQ(f[1], 0);
    }
    // AdaptationIntegrationTest.cpp:62-128: split then merge through the engine
    {
        Mesh m(dev, 1024);
        m.upload({0}, {0}, {0}, {0}, {0}, {1}, {0});
        AdaptationEngine eng(dev, cfg);
        eng.adapt(m);
        EXPECT_EQ(m.size(), (size_t)8);
        std::vector<int32_t> fl(8, -1);
        check(dev.get(), fl_memcpy_h2d(dev.get(), m.raw().flags, fl.data(), 32), "flags");
        eng.adapt(m);
        EXPECT_EQ(m.size(), (size_t)1);
        EXPECT_EQ((int)m.read(m.raw().level)[0], 0);
    }
    // RadixSort::sortByKey in every shape: the same stable order (ties keep input order)
    {
        const size_t n = 100003;
        std::vector<uint64_t> k(n);
        std::vector<uint32_t> v(n);
        uint64_t s = 88172645463325252ull;
        for (size_t i = 0; i < n; ++i) {
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            k[i] = s % 5000;  // many ties
            v[i] = (uint32_t)i;
        }
        uint64_t* dk = nullptr;
        uint32_t* dv = nullptr;
        check(dev.get(), fl_device_alloc(dev.get(), n * 8, (void**)&dk), "alloc");
        check(dev.get(), fl_device_alloc(dev.get(), n * 4, (void**)&dv), "alloc");
        hashmap::RadixSort rs(dev);
        std::vector<uint64_t> k0(n);
        std::vector<uint32_t> v0(n);
        const int shapes[4][2] = {{8, 256}, {8, 512}, {9, 256}, {9, 512}};
        for (int t = 0; t < 4; ++t) {
            rs.setShape(shapes[t][0], shapes[t][1]);
            check(dev.get(), fl_memcpy_h2d(dev.get(), dk, k.data(), n * 8), "h2d");
            check(dev.get(), fl_memcpy_h2d(dev.get(), dv, v.data(), n * 4), "h2d");
            rs.sortByKey(dk, dv, n, 0, 13);
            std::vector<uint64_t> kk(n);
            std::vector<uint32_t> vv(n);
            check(dev.get(), fl_memcpy_d2h(dev.get(), kk.data(), dk, n * 8), "d2h");
            check(dev.get(), fl_memcpy_d2h(dev.get(), vv.data(), dv, n * 4), "d2h");
            bool stable = true;
            for (size_t i = 1; i < n; ++i)
                stable = stable && (kk[i - 1] < kk[i] || (kk[i - 1] == kk[i] && vv[i - 1] < vv[i]));
            EXPECT_TRUE(stable);
            if (t == 0) { k0 = kk; v0 = vv; }
            EXPECT_TRUE(kk == k0 && vv == v0);
        }
        rs.setShape(8, 256);
        bool refused = false;
        try { rs.setShape(10, 256); } catch (const FluidLoomError&) { refused = true; }
        EXPECT_TRUE(refused);
        fl_device_free(dev.get(), dk);
        fl_device_free(dev.get(), dv);
    }
    // a pool step through the runtime nodes
    {
        fl_lbm_case c{};
        c.ext[0] = c.ext[1] = c.ext[2] = 2;
        int bc[6] = {1, 1, 1, 1, 1, 2};
        for (int k = 0; k < 6; ++k) c.bc[k] = bc[k];
        c.wall_u[0] = 0.05f;
        c.tau0 = 0.56f;
        c.max_level = 1;
        c.refine_frac = 0.5f;
        c.coarsen_frac = 0.1f;
        runtime::BrickPool pool(dev, {c});
        runtime::LbmStepNode step(pool, 4);
        runtime::AdaptMeshNode adapt(pool);
        step.execute();
        adapt.execute();
        step.execute();
        dev.finish();
        EXPECT_TRUE(pool.info().num_bricks >= 8);
        // a solid block through the mask: fewer fluid updates, the same words back
        const uint64_t lups = pool.info().fluid_lups_per_step;
        std::vector<uint32_t> bits(16 * 16 * 16 / 32, 0u);
        for (int z = 4; z < 8; ++z)
            for (int y = 4; y < 8; ++y)
                for (int x = 4; x < 8; ++x) {
                    const int i = (z * 16 + y) * 16 + x;
                    bits[i >> 5] |= 1u << (i & 31);
                }
        pool.setSolidMask(0, 0, bits);
        std::vector<uint32_t> back;
        EXPECT_EQ(pool.solidMask(0, &back), 0);
        EXPECT_TRUE(back == bits);
        EXPECT_TRUE(pool.info().fluid_lups_per_step < lups);
        step.execute();
        pool.setSolidMask(0, 0, {});
        EXPECT_EQ(pool.solidMask(0, nullptr), -1);
        EXPECT_EQ(pool.info().fluid_lups_per_step, lups);
        // the populations bound the reference's way: a 19-component field of the SOA manager
        // whose component pointers a kernel node binds (KernelNode::bindField); equal to the
        // downloaded populations, and writes through the field reach the pool
        {
            // one more level-0 step: an odd count, so level 0's current populations sit in buffer B
            check(dev.get(), fl_pool_step(dev.get(), pool.get(), 1), "step");
            fields::SOAFieldManager soa(dev);
            fields::FieldHandle h = pool.populationsField("f");
            const size_t n = pool.info().num_bricks;
            EXPECT_EQ(soa.numCells(h), n * 512);
            std::vector<float> all(19 * n * 512), comp(n * 512);
            check(dev.get(), fl_pool_download(dev.get(), pool.get(), nullptr, nullptr, nullptr, nullptr, nullptr,
                                              all.data()), "download");
            bool same = true;
            for (int q = 0; q < 19; ++q) {
                check(dev.get(), fl_memcpy_d2h(dev.get(), comp.data(), soa.getDevicePtr(h, (uint16_t)q),
                                               comp.size() * 4), "field read");
                for (size_t i = 0; i < comp.size(); ++i) same = same && comp[i] == all[q * n * 512 + i];
            }
            EXPECT_TRUE(same);
            const float v = 0.25f;
            check(dev.get(), fl_memcpy_h2d(dev.get(), soa.getDevicePtr(h, 3), &v, 4), "field write");
            check(dev.get(), fl_pool_download(dev.get(), pool.get(), nullptr, nullptr, nullptr, nullptr, nullptr,
                                              all.data()), "download");
            EXPECT_EQ(all[3 * n * 512], v);
        }
        // the same three operations as an execution graph (test_hazard_analyzer.cpp / 
        // test_topological_scheduler.cpp shapes): hazards chain them, the order is A, B, C
        runtime::BrickPool pool2(dev, {c});
        runtime::dependency::DependencyGraph g(dev.get());
        int64_t a = g.addNode(FL_NODE_LBM_STEP, "lbm", "f", "f", -1, pool2.get(), 4);
        int64_t b = g.addNode(FL_NODE_ADAPT_MESH, "adapt", "f,mesh", "f,mesh", -1, pool2.get());
        int64_t d = g.addNode(FL_NODE_LBM_STEP, "lbm2", "f,mesh", "f", -1, pool2.get(), 4);
        auto hz = g.analyzeNodes();
        EXPECT_TRUE(hz.size() >= 2);
        g.build();
        auto order = g.getTopologicalOrder();
        EXPECT_EQ(order.size(), (size_t)3);
        EXPECT_EQ((int64_t)order[0], a);
        EXPECT_EQ((int64_t)order[1], b);
        EXPECT_EQ((int64_t)order[2], d);
        runtime::scheduler::TopologicalScheduler sched(g, true);
        EXPECT_TRUE(sched.execute());
        dev.finish();
        EXPECT_EQ(pool2.info().num_bricks, pool.info().num_bricks);
        // a cycle is rejected (test_topological_scheduler.cpp:103-126)
        runtime::dependency::DependencyGraph cyc;
        int64_t x = cyc.addNode(FL_NODE_KERNEL, "A", "", "");
        int64_t y = cyc.addNode(FL_NODE_KERNEL, "B", "", "");
        cyc.addEdge(x, y);
        cyc.addEdge(y, x);
        bool threw = false;
        try {
            cyc.build();
        } catch (const FluidLoomError&) {
            threw = true;
        }
        EXPECT_TRUE(threw);
    }
    if (failures) {
        std::printf("%d FAILURES\n", failures);
        return 1;
    }
    std::printf("ALL PASSED\n");
    return 0;
}
