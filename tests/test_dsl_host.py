"""The .fl subset on the host: tokens and precedence of the reference's
expression grammar (FluidLoomExpressionParser.g4), statement forms of the
kernel/simulation grammars, the mapping of scripts onto case parameters, and the
reference's own benchmark scripts (when the reference tree is present)."""
import os

import pytest

from fluidloom_gb300 import dsl
from oracle.build import REF_ROOT

SCEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fluidloom_gb300", "scenarios")
REF_BENCH = os.path.join(REF_ROOT, "benchmarks")


def ev(src, **names):
    e = dsl.Parser(src).expression()
    return dsl.evaluate(e, dsl.Env(names))


def test_expression_precedence_and_operators():
    assert ev("2 + 3 * 4 ** 2") == 50
    assert ev("(2 + 3) * 4") == 20
    assert ev("-2 ** 2") == 4          # unary binds tighter than ** (unaryExpression CARET unaryExpression)
    assert bool(ev("7 % 4 == 3 && !false"))
    assert bool(ev("1 < 2 || 4 / 2 > 3")) and not bool(ev("1 > 2 || 4 / 2 > 3"))
    assert ev('"step " + t + "!"', t=40) == "step 40!"
    assert abs(ev("sqrt(pow(3, 2) + 4 ** 2)") - 5.0) < 1e-12
    v = ev("(1.0, 2.0, 3.0)")
    assert list(v) == [1.0, 2.0, 3.0]
    assert ev("distance((0.0, 0.0, 0.0), (3.0, 4.0, 0.0))") == 5.0


def test_comments_ranges_and_else_if():
    tree = dsl.parse("""
        // line comment
        /* block
           comment */
        field a: scalar  # trailing comment
        time_loop: {
            for i in 0..num_cells { if a[i] > 1 { x = 1 } else if a[i] < 0 { x = 2 } else { x = 3 } }
        }""")
    loop = tree["blocks"]["time_loop"][0]
    assert loop[0] == "for" and loop[2] == ("num", 0) and loop[3] == ("name", "num_cells")
    branch = loop[4][0]
    assert branch[0] == "if" and branch[3][0][0] == "if"


def test_parse_errors_name_the_line():
    with pytest.raises(dsl.ParseError, match="line 3"):
        dsl.parse("field a: scalar\ntime_loop: {\n  run (\n}")
    with pytest.raises(dsl.ParseError, match="no GB300 implementation"):
        dsl.Scenario(dsl.parse("time_loop: { run make_coffee() }"))


def test_kernel_definition_clauses():
    tree = dsl.parse("""
        kernel relax: { reads: f, rho writes: g halo: 1 execution_mask: "cell_state == 0"
                        script: | g[i] = f[i] * 0.5 | }
        time_loop: { run lbm_step() }""")
    k = tree["kernels"]["relax"]
    assert k["reads"] == ["f", "rho"] and k["writes"] == ["g"] and k["halo"] == 1 and k["mask"] == "cell_state == 0"
    assert k["body"][0][0] == "assign"


def test_example_scenarios_map_to_cases():
    cav = dsl.Scenario(dsl.parse(open(os.path.join(SCEN, "cavity.fl")).read()))
    assert cav.kind == "cavity" and cav.lid == 0.05 and cav.regrid_every == 20
    assert cav.rule == {"field": "vorticity", "refine": 0.5, "coarsen": 0.1}
    c = cav.case()
    assert list(c.ext) == [4, 4, 4] and c.max_level == 2 and abs(c.wall_u[0] - 0.05) < 1e-7
    sph = dsl.Scenario(dsl.parse(open(os.path.join(SCEN, "sphere.fl")).read()))
    assert sph.kind == "channel" and sph.sphere == ((32.0, 32.0, 32.0), 8.0) and sph.regrid_every == 25
    c = sph.case()
    assert list(c.ext) == [16, 8, 8] and c.has_sphere == 1 and abs(c.inlet_u[0] - 0.04) < 1e-7


@pytest.mark.skipif(not os.path.isdir(REF_BENCH), reason="reference tree not present")
def test_reference_benchmark_scripts_parse_and_map():
    cav = dsl.Scenario(dsl.parse(open(os.path.join(REF_BENCH, "lid_driven_cavity.fl")).read()))
    assert cav.kind == "cavity" and cav.lid == 0.1 and cav.regrid_every == 100 and cav.note
    sph = dsl.Scenario(dsl.parse(open(os.path.join(REF_BENCH, "flow_past_sphere.fl")).read()))
    assert sph.kind == "channel" and sph.inlet == (0.1, 0.0, 0.0) and sph.regrid_every == 50
    assert sph.rule["field"] == "q_criterion"


def test_placed_solids_map_to_mask_geometry(tmp_path):
    from fluidloom_gb300 import geometry as G
    sc = dsl.Scenario(dsl.parse(open(os.path.join(SCEN, "obstacles.fl")).read()), ext=(8, 8, 8), max_level=2)
    assert sc.kind == "channel" and sc.sphere is None and sc.mask_level == 2
    assert [g["type"] for g in sc.solids] == ["box", "cylinder"]
    assert sc.case().has_sphere == 0
    (box, t0), (cyl, t1) = sc.solid_geometries()
    assert t0 is None and t1 is None
    assert box.type == G.BOX and list(box.translate) == [96.0, 120.0, 128.0] and list(box.scale) == [4.0] * 3
    assert (box.width, box.height, box.length) == (6.0, 10.0, 8.0)
    assert cyl.type == G.CYLINDER and cyl.radius == 3.0 and list(cyl.translate) == [176.0, 128.0, 96.0]
    # a second sphere, a scaled sphere and an STL file become mask geometry; implicit functions are refused
    G.write_stl(str(tmp_path / "tet.stl"), [[0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, 0, 0, 0, 1, 1, 0, 0],
                                            [0, 0, 0, 0, 1, 0, 0, 0, 1], [1, 0, 0, 0, 0, 1, 0, 1, 0]])
    src = """
        geometry a { type: sphere  radius: 4.0  translate: (16.0, 16.0, 16.0) }
        geometry b { type: sphere  radius: 2.0  translate: (40.0, 16.0, 16.0) }
        geometry c { type: stl  source: "tet.stl"  scale: (8.0, 8.0, 8.0)  translate: (50.0, 20.0, 20.0) }
        initial_condition: { place_geometry(a)  place_geometry(b)  place_geometry(c) }
        time_loop: { run lbm_step()  run apply_inlet_velocity(velocity_inlet = (0.03, 0.0, 0.0)) }"""
    sc = dsl.Scenario(dsl.parse(src), ext=(8, 4, 4), max_level=1, base_dir=str(tmp_path))
    assert sc.sphere == ((16.0, 16.0, 16.0), 4.0) and [g["type"] for g in sc.solids] == ["sphere", "stl"]
    assert sc.mask_level == 1 and sc.case().has_sphere == 1
    (_, none), (stl, tris) = sc.solid_geometries()
    assert none is None and stl.type == G.STL and tris.shape == (4, 9) and list(stl.scale) == [16.0] * 3
    with pytest.raises(dsl.ParseError, match="not placed"):
        dsl.Scenario(dsl.parse("initial_condition: { place_geometry(type = \"implicit\") }"))


def test_expression_parser_agrees_with_python_on_random_arithmetic():
    """Random integer expressions over + - * % and ( ): left-associative binary operators
    with * and % above + and -, as FluidLoomExpressionParser.g4 orders them (and Python)."""
    pytest.importorskip("hypothesis")
    from hypothesis import given, settings, strategies as st

    atoms = st.integers(0, 9).map(str) | st.integers(1, 9).map(lambda v: "(-%d)" % v)

    def extend(children):
        return (st.tuples(children, st.sampled_from(["+", "-", "*", "%"]), children)
                .filter(lambda t: t[1] != "%" or t[2] not in ("0", "(0)"))
                .map(lambda t: "%s %s %s" % t) | children.map(lambda c: "(%s)" % c))

    @settings(max_examples=300, deadline=None)
    @given(st.recursive(atoms, extend, max_leaves=12))
    def check(src):
        try:
            want = eval(src)
        except ZeroDivisionError:
            return
        assert ev(src) == want, src

    check()
