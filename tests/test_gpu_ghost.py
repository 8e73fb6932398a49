"""GPU ghost pack/unpack, trilinear interpolation, restriction, split/merge
entry points and blob flags vs the oracle."""
import ctypes

import numpy as np
import pytest

from tests import _oracle as O

pytestmark = pytest.mark.gpu


def D(ctx, a):
    from fluidloom_gb300 import DeviceArray
    return DeviceArray.from_host(ctx, np.ascontiguousarray(a))


def E(ctx, shape, dt):
    from fluidloom_gb300 import DeviceArray
    return DeviceArray(ctx, shape, dt)


def test_pack_unpack_fields_roundtrip(ctx):
    # test_halo_exchanger.cpp:82-123: pack then unpack is the identity
    rng = np.random.default_rng(0)
    f = rng.standard_normal(10007).astype(np.float32)
    df, buf, back = D(ctx, f), E(ctx, (4 * 10007 + 64,), np.uint8), E(ctx, (10007,), np.float32)
    ctx.call("fl_pack_fields", df.ptr, buf.ptr, 10007, 64)
    ctx.call("fl_unpack_fields", buf.ptr, back.ptr, 10007, 64)
    np.testing.assert_array_equal(back.to_host(), f)
    np.testing.assert_array_equal(buf.to_host()[64:].view(np.float32), f)


@pytest.mark.parametrize("C,m", [(19, 700), (1, 1001), (7, 333), (32, 9), (33, 77), (70, 130)])
def test_pack_unpack_halo(ctx, C, m):
    """Rows narrower than a warp (several per warp), exactly a warp, and wider;
    row counts that leave partial rounds."""
    rng = np.random.default_rng(C)
    n = 5000
    f = rng.standard_normal((n, C)).astype(np.float32)
    idx = rng.choice(n, m, replace=False).astype(np.uint32)
    df, di, pk = D(ctx, f), D(ctx, idx), E(ctx, (m, C), np.float32)
    ctx.call("fl_pack_halo", df.ptr, C, di.ptr, m, pk.ptr)
    np.testing.assert_array_equal(pk.to_host(), f[idx])
    g = np.zeros_like(f)
    dg = D(ctx, g)
    ctx.call("fl_unpack_halo", pk.ptr, C, di.ptr, m, dg.ptr)
    g[idx] = f[idx]
    np.testing.assert_array_equal(dg.to_host(), g)


def test_interp_trilinear_vs_oracle(ctx):
    from fluidloom_gb300.amr import AdaptConfig, Mesh
    cols = O.random_octree(31, ext=(1, 1, 1), rounds=4, max_level=6, frac=0.3, balanced=True)
    n = len(cols["x"])
    C = 7
    rng = np.random.default_rng(2)
    f = rng.standard_normal((n, C)).astype(np.float32)
    # queries: children of every cell (fine coords at level + 1)
    fx = np.repeat(cols["x"] * 2, 8) + np.tile(np.arange(8) & 1, n)
    fy = np.repeat(cols["y"] * 2, 8) + np.tile((np.arange(8) >> 1) & 1, n)
    fz = np.repeat(cols["z"] * 2, 8) + np.tile(np.arange(8) >> 2, n)
    fl = np.repeat(cols["level"].astype(np.uint8) + 1, 8).astype(np.uint8)
    m, keep = O.mesh_struct(cols)
    want = np.zeros((len(fx), C), np.float32)
    fxyz = [np.ascontiguousarray(a, np.int32) for a in (fx, fy, fz)]
    O.load().or_interp_trilinear(ctypes.byref(m), ctypes.byref(O.domain(max_level=7)), O.ptr(f), C,
                                 *[O.ptr(a) for a in fxyz], O.ptr(fl), len(fx), O.ptr(want))
    gm = Mesh(ctx, cols)
    dfs = [D(ctx, a) for a in fxyz] + [D(ctx, fl)]
    df, out = D(ctx, f), E(ctx, (len(fx), C), np.float32)
    ctx.call("fl_interp_trilinear", ctypes.byref(gm.m), ctypes.byref(AdaptConfig.make(max_level=7)), df.ptr, C,
             dfs[0].ptr, dfs[1].ptr, dfs[2].ptr, dfs[3].ptr, len(fx), out.ptr)
    np.testing.assert_array_equal(out.to_host(), want)
    assert np.abs(want).sum() > 0


@pytest.mark.parametrize("C,G", [(5, 300), (19, 301), (1, 257), (32, 33), (40, 97)])
def test_restrict_groups_vs_oracle(ctx, C, G):
    """Rows narrower than a warp, exactly a warp and wider; odd group counts."""
    rng = np.random.default_rng(3 + C)
    n = 8 * G + 100
    f = rng.standard_normal((n, C)).astype(np.float32)
    mem = rng.choice(n, G * 8, replace=False).astype(np.uint32)
    for rule in (0, 1):
        want = np.zeros((G, C), np.float32)
        O.load().or_restrict_groups(O.ptr(f), C, O.ptr(mem), G, rule, O.ptr(want))
        df, dm, out = D(ctx, f), D(ctx, mem), E(ctx, (G, C), np.float32)
        ctx.call("fl_restrict_groups", df.ptr, C, dm.ptr, G, rule, out.ptr)
        np.testing.assert_array_equal(out.to_host(), want)


def test_split_merge_entry_points_vs_oracle(ctx):
    from fluidloom_gb300.amr import AdaptConfig, Mesh
    cols = O.random_octree(40, ext=(1, 1, 1), rounds=3, max_level=6, frac=0.3, balanced=True)
    rng = np.random.default_rng(4)
    n = len(cols["x"])
    cols["flags"] = rng.choice([-1, 0, 1], n, p=[0.6, 0.2, 0.2]).astype(np.int32)
    C = 3
    f = rng.standard_normal((n, C)).astype(np.float32)
    cfg = AdaptConfig.make(max_level=6, min_level=1)
    m = Mesh(ctx, cols)
    ch = Mesh(ctx, {k: np.zeros(8 * n, np.int32 if k in ("x", "y", "z", "flags") else np.uint8 if k in ("level", "state") else np.uint32)
                    for k in ("x", "y", "z", "level", "state", "flags", "material")}, capacity=8 * n)
    df, cf, p2c = D(ctx, f), E(ctx, (8 * n, C), np.float32), E(ctx, (n,), np.uint32)
    nc = ctypes.c_size_t()
    ctx.call("fl_split", ctypes.byref(m.m), ctypes.byref(cfg), df.ptr, C, ctypes.byref(ch.m), cf.ptr, p2c.ptr,
             ctypes.byref(nc))
    pred = (cols["flags"] > 0) & (cols["state"] == 0) & (cols["level"] < 6)
    assert nc.value == 8 * pred.sum()
    got = ch.download()
    par = np.nonzero(pred)[0]
    ci = np.arange(8)
    np.testing.assert_array_equal(got["x"], (np.repeat(cols["x"][par] * 2, 8) + np.tile(ci & 1, len(par))))
    np.testing.assert_array_equal(got["level"], np.repeat(cols["level"][par] + 1, 8))
    np.testing.assert_array_equal(cf.to_host()[:nc.value], np.repeat(f[par], 8, axis=0))
    p = p2c.to_host()
    assert (p[~pred] == 0xFFFFFFFF).all() and (p[par] == np.arange(len(par)) * 8).all()
    # merge: groups and restricted fields equal the oracle regrid's parents
    want, wst, wf, src, kind, members, _ = O.adapt(dict(cols, flags=np.where(cols["flags"] < 0, -1, 0).astype(np.int32)),
                                                   dict(max_level=6, min_level=1, balance_mode=0,
                                                        max_balance_iterations=10, enforce_balance=0,
                                                        averaging_rule=0), O.domain(max_level=6), f, C)
    pm = Mesh(ctx, {k: np.zeros(n, np.int32 if k in ("x", "y", "z", "flags") else np.uint8 if k in ("level", "state") else np.uint32)
                    for k in ("x", "y", "z", "level", "state", "flags", "material")}, capacity=n)
    mcols = dict(cols, flags=np.where(cols["flags"] < 0, -1, 0).astype(np.int32))
    m2 = Mesh(ctx, mcols)
    pf, gid = E(ctx, (n, C), np.float32), E(ctx, (n,), np.uint32)
    npar = ctypes.c_size_t()
    ctx.call("fl_merge", ctypes.byref(m2.m), ctypes.byref(cfg), df.ptr, C, ctypes.byref(pm.m), pf.ptr, gid.ptr,
             ctypes.byref(npar))
    assert npar.value == wst.num_groups
    G = npar.value
    mem = members.reshape(-1, 8)
    gp = pm.download()
    np.testing.assert_array_equal(gp["x"], cols["x"][mem[:, 0]] >> 1)
    np.testing.assert_array_equal(gp["level"], cols["level"][mem[:, 0]] - 1)
    want_f = np.zeros((G, C), np.float32)
    O.load().or_restrict_groups(O.ptr(f), C, O.ptr(np.ascontiguousarray(members)), G, 0, O.ptr(want_f))
    np.testing.assert_array_equal(pf.to_host()[:G], want_f)


def test_blob_flags_vs_oracle(ctx):
    from fluidloom_gb300.amr import Mesh
    cols = O.random_octree(50, ext=(1, 1, 1), rounds=2, max_level=7, frac=0.2, balanced=True, start_level=5)
    blobs = O.gaussian_blobs(7)
    want = O.blob_flags(cols, blobs, 0.05, 0.5, 7)
    m = Mesh(ctx, cols)
    ctx.call("fl_flags_from_blobs", ctypes.byref(m.m), blobs.ctypes.data_as(ctypes.c_void_p), len(blobs),
             ctypes.c_float(0.05), ctypes.c_float(0.5), 7)
    np.testing.assert_array_equal(m.download()["flags"], want)
    assert (want == 1).any() and (want == -1).any()
