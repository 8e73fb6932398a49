"""The .fl subset on the host: tokens and precedence of the reference's
expression grammar (FluidLoomExpressionParser.g4), statement forms of the
kernel/simulation grammars, the mapping of scripts onto case parameters, and the
reference's own benchmark scripts (when the reference tree is present)."""
import os

import pytest

from fluidloom_gb300 import dsl

SCEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fluidloom_gb300", "scenarios")
REF_BENCH = "/root/reference/benchmarks"


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
