"""`.fl` simulation scripts: a hand-written parser for the subset of the
reference's simulation grammar that drives the AMR lattice-Boltzmann path, and a
runner with a real time loop.

The grammar followed is src/parsing/grammars/FluidLoomSimulationParser.g4
(imports, `field` declarations, `geometry` blocks, `initial_condition`,
`time_loop`, `final_output` blocks of script statements), with the statement
and expression rules of FluidLoomKernelParser.g4 / FluidLoomExpressionParser.g4
and the tokens of the three lexers (`**` is the power operator, `..` a range,
`#`, `//` and `/* */` comments).  Two lenient extensions accept what the
reference's own benchmark scripts write: typed local declarations
(`float d = ...`, `vec3 p = ...`) and keyword-argument `place_geometry(...)`.

How a script maps onto the engine -- the reference's SimulationBuilder does the
same by kernel name (src/parsing/SimulationBuilder.cpp:192-363):
  * `run lbm_*` statements of one time-loop iteration are one fused
    collide-stream step of the pool; `run apply_*` statements select the
    boundary conditions (`apply_moving_lid(velocity_lid = v)` -> lid velocity,
    `apply_inlet_velocity(velocity_inlet = vec3(...))` -> inlet, `apply_outlet_*`
    -> zero-gradient outlet, `apply_*bounce_back*` -> walls / sphere);
  * `run compute_vorticity` / `compute_q_criterion` name the refinement
    indicator (|curl u| per brick, computed by the regrid itself); a per-cell loop
    setting `refine_flag[i]` from `indicator > A` / `< B` gives the refine and
    coarsen thresholds, read as fractions of the case's maximum (the reading the
    benchmark configuration states for these loops);
  * `if timestep % N == 0 { adapt_mesh() ... }` regrids every N steps (any
    period-guarded `print` / `write_vtk` / `write_hdf5` fires with the same rule);
  * in `initial_condition`, uniform `density[i]` / `velocity[i]` assignments set
    the initial state, `place_geometry` the case's sphere (the first unscaled
    one) or solid-mask geometry (further spheres, boxes, cylinders, STL meshes:
    voxelised on the GPU into the case's mask at --mask-level, the mesh then
    pre-refined around them), and a per-cell loop writing
    `refine_flag[i] = k` under a condition (evaluated per brick at its centre,
    `cell_position(i)`) followed by `adapt_mesh()` pre-refines up to k levels;
  * `write_vtk(fields..., path)` writes a VTK PolyData file (fluidloom_gb300.io),
    `write_hdf5(..., path)` a snapshot (.npz: there is no HDF5 library here).
The lattice is always D3Q19 (a `d2q9` import runs the three-dimensional case).
Unknown `run` kernels are an error: there is no generic kernel compiler.

  python -m fluidloom_gb300.dsl script.fl --steps 200 [--ext 4 4 4] [--max-level 2]
"""
import argparse
import json
import math
import os
import re
import time

import numpy as np

# ---------------------------------------------------------------- lexer

_TOKEN = re.compile(r"""
    (?P<ws>[ \t\r\n]+)
  | (?P<comment>\#[^\n]*|//[^\n]*|/\*.*?\*/)
  | (?P<float>\d+\.\d+(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)
  | (?P<int>\d+)
  | (?P<string>"(?:[^"\\\n]|\\.)*")
  | (?P<op>\*\*|\.\.|==|!=|<=|>=|&&|\|\||[-+*/%()\[\]{},.:;<>=!|])
  | (?P<ident>[A-Za-z_][A-Za-z0-9_]*)
""", re.S | re.X)


class ParseError(Exception):
    """A script the subset cannot read (line and token in the message)."""


def tokenize(src):
    out, pos, line = [], 0, 1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise ParseError("line %d: unexpected character %r" % (line, src[pos]))
        kind, text = m.lastgroup, m.group()
        if kind not in ("ws", "comment"):
            out.append((kind, text, line))
        line += text.count("\n")
        pos = m.end()
    out.append(("eof", "", line))
    return out


# ---------------------------------------------------------------- parser

_BLOCKS = ("initial_condition", "time_loop", "final_output")


class Parser:
    def __init__(self, src):
        self.t = tokenize(src)
        self.i = 0

    # token helpers
    def peek(self, k=0):
        return self.t[min(self.i + k, len(self.t) - 1)]

    def at(self, text, k=0):
        tok = self.peek(k)
        return tok[0] in ("op", "ident") and tok[1] == text

    def take(self, text=None, kind=None):
        tok = self.peek()
        if text is not None and not self.at(text):
            raise ParseError("line %d: expected %r, found %r" % (tok[2], text, tok[1]))
        if kind is not None and tok[0] != kind:
            raise ParseError("line %d: expected %s, found %r" % (tok[2], kind, tok[1]))
        self.i += 1
        return tok

    def opt(self, text):
        if self.at(text):
            self.i += 1
            return True
        return False

    # file
    def parse(self):
        f = {"imports": [], "fields": [], "geometries": {}, "kernels": {}, "blocks": {}}
        while not self.peek()[0] == "eof":
            if self.opt("import"):
                f["imports"].append(self.take(kind="string")[1][1:-1])
                self.opt(";")
            elif self.opt("field"):
                name = self.take(kind="ident")[1]
                self.take(":")
                f["fields"].append((name, self.take(kind="ident")[1]))
                self.opt(";")
            elif self.opt("geometry"):
                name = self.take(kind="ident")[1]
                f["geometries"][name] = self.geometry_props()
            elif self.opt("kernel"):
                k = self.kernel_def()
                f["kernels"][k["name"]] = k
            elif self.peek()[1] in _BLOCKS:
                name = self.take()[1]
                self.take(":")
                f["blocks"][name] = self.block()
            else:
                tok = self.peek()
                raise ParseError("line %d: unexpected %r at file level" % (tok[2], tok[1]))
        return f

    def geometry_props(self):
        props = {}
        self.take("{")
        while not self.opt("}"):
            key = self.take(kind="ident")[1]
            self.take(":")
            if self.at("("):
                props[key] = self.expression()
            else:
                tok = self.take()
                props[key] = float(tok[1]) if tok[0] in ("int", "float") else tok[1].strip('"')
            self.opt(";")
        return props

    def kernel_def(self):
        name = self.take(kind="ident")[1]
        self.take(":")
        self.take("{")
        k = {"name": name, "reads": [], "writes": [], "halo": 0, "mask": None, "body": []}
        while not self.at("script"):
            if self.opt(","):
                continue
            key = self.take(kind="ident")[1]
            self.take(":")
            if key in ("reads", "writes"):
                k[key].append(self.take(kind="ident")[1])
                while self.at(",") and self.peek(1)[0] == "ident" and not self.at(":", 2):
                    self.take(",")
                    k[key].append(self.take(kind="ident")[1])
            elif key == "halo":
                k["halo"] = int(self.take(kind="int")[1])
            elif key == "execution_mask":
                k["mask"] = self.take(kind="string")[1][1:-1]
            else:
                raise ParseError("kernel %s: unknown clause %s" % (name, key))
        self.take("script")
        self.take(":")
        self.take("|")
        while not self.opt("|"):
            k["body"].append(self.statement())
        self.take("}")
        return k

    def block(self):
        self.take("{")
        out = []
        while not self.opt("}"):
            out.append(self.statement())
        return out

    def body(self):
        return self.block() if self.at("{") else [self.statement()]

    # statements
    def statement(self):
        tok = self.peek()
        w = tok[1]
        if tok[0] != "ident":
            raise ParseError("line %d: unexpected %r" % (tok[2], w))
        if w == "run":
            self.take()
            name = self.take(kind="ident")[1]
            args = self.call_args()
            self.opt(";")
            return ("run", name, args, tok[2])
        if w in ("adapt_mesh", "rebalance_mesh") and self.at("(", 1):
            self.take()
            self.take("(")
            self.take(")")
            self.opt(";")
            return ("adapt",) if w == "adapt_mesh" else ("rebalance",)
        if w in ("write_vtk", "write_hdf5") and self.at("(", 1):
            self.take()
            args = self.call_args()
            self.opt(";")
            return ("write", w, args)
        if w == "print" and self.at("(", 1):
            self.take()
            self.take("(")
            e = self.expression()
            self.take(")")
            self.opt(";")
            return ("print", e)
        if w == "place_geometry" and self.at("(", 1):
            self.take()
            args = self.call_args()
            self.opt(";")
            return ("place", args)
        if w in ("reduce_sum", "reduce_min", "reduce_max"):
            self.take()
            self.take("(")
            e = self.expression()
            self.take(")")
            self.opt(";")
            return ("reduce", w, e)
        if w == "for":
            self.take()
            var = self.take(kind="ident")[1]
            self.take("in")
            lo = self.expression()
            self.take("..")
            hi = self.expression()
            return ("for", var, lo, hi, self.body())
        if w == "while":
            self.take()
            cond = self.expression()
            return ("while", cond, self.body())
        if w == "if":
            self.take()
            cond = self.expression()
            then = self.body()
            other = []
            if self.opt("else"):
                other = self.body()
            return ("if", cond, then, other)
        # typed local declaration: <type> <name> = expr
        if self.peek(1)[0] == "ident" and self.at("=", 2):
            ty = self.take()[1]
            name = self.take()[1]
            self.take("=")
            e = self.expression()
            self.opt(";")
            return ("decl", ty, name, e)
        # assignment: name(.member)?([index])? = expr
        save = self.i
        name = self.take()[1]
        member = None
        if self.at(".") and self.peek(1)[0] == "ident":
            self.take(".")
            member = self.take()[1]
        index = None
        if self.opt("["):
            index = self.expression()
            self.take("]")
        if self.opt("="):
            e = self.expression()
            self.opt(";")
            return ("assign", name, member, index, e)
        self.i = save
        e = self.expression()
        self.opt(";")
        return ("expr", e)

    def call_args(self):
        self.take("(")
        args = []
        while not self.opt(")"):
            kw = None
            if self.peek()[0] == "ident" and self.at("=", 1):
                kw = self.take()[1]
                self.take("=")
            args.append((kw, self.expression()))
            if not self.at(")"):
                self.take(",")
        return args

    # expressions (FluidLoomExpressionParser.g4 precedence)
    def expression(self):
        return self.binary(0)

    _LEVELS = [("||",), ("&&",), ("==", "!="), ("<", "<=", ">", ">="), ("+", "-"), ("*", "/", "%")]

    def binary(self, lvl):
        if lvl == len(self._LEVELS):
            return self.power()
        e = self.binary(lvl + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self._LEVELS[lvl]:
            op = self.take()[1]
            e = ("bin", op, e, self.binary(lvl + 1))
        return e

    def power(self):
        e = self.unary()
        if self.opt("**"):
            e = ("bin", "**", e, self.unary())
        return e

    def unary(self):
        if self.peek()[0] == "op" and self.peek()[1] in ("+", "-", "!"):
            op = self.take()[1]
            return ("un", op, self.unary())
        return self.postfix()

    def postfix(self):
        e = self.primary()
        while True:
            if self.at("(") and e[0] == "name":
                e = ("call", e[1], self.call_args())
            elif self.at("["):
                self.take("[")
                e = ("index", e, self.expression())
                self.take("]")
            elif self.at(".") and self.peek(1)[0] == "ident":
                self.take(".")
                e = ("member", e, self.take()[1])
            else:
                return e

    def primary(self):
        kind, text, line = self.peek()
        if kind == "int":
            self.take()
            return ("num", int(text))
        if kind == "float":
            self.take()
            return ("num", float(text))
        if kind == "string":
            self.take()
            return ("str", bytes(text[1:-1], "utf-8").decode("unicode_escape"))
        if kind == "ident":
            self.take()
            if text in ("true", "false"):
                return ("num", text == "true")
            if text == "lambda":
                params = []
                while not self.opt(":"):
                    params.append(self.take(kind="ident")[1])
                    self.opt(",")
                return ("lambda", params, self.expression())
            return ("name", text)
        if self.opt("("):
            items = [self.expression()]
            while self.opt(","):
                items.append(self.expression())
            self.take(")")
            return items[0] if len(items) == 1 else ("vec", items)
        raise ParseError("line %d: unexpected %r in an expression" % (line, text))


def parse(src):
    return Parser(src).parse()


# ---------------------------------------------------------------- evaluation

class Env:
    """Values of an expression evaluation: scalars, numpy arrays (per-brick
    vectorised loops), 3-vectors (arrays of shape (..., 3)) and strings."""

    def __init__(self, names=None, cell=None):
        self.names = dict(names or {})
        self.cell = cell  # per-brick arrays for cell_position(i) in vectorised loops


def _vec(*xs):
    return np.stack(np.broadcast_arrays(*[np.asarray(x, np.float64) for x in xs]), -1)


def _fmt(v):
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        return repr(float(v))
    return str(v)


def evaluate(e, env):
    k = e[0]
    if k == "num" or k == "str":
        return e[1]
    if k == "name":
        if e[1] in env.names:
            return env.names[e[1]]
        raise ParseError("unknown name %r" % e[1])
    if k == "vec":
        return _vec(*[evaluate(x, env) for x in e[1]])
    if k == "un":
        v = evaluate(e[2], env)
        return -v if e[1] == "-" else (v if e[1] == "+" else np.logical_not(v))
    if k == "bin":
        a, b = evaluate(e[2], env), evaluate(e[3], env)
        op = e[1]
        if op == "+" and (isinstance(a, str) or isinstance(b, str)):
            return _fmt(a) + _fmt(b)
        if op == "&&":
            return np.logical_and(a, b)
        if op == "||":
            return np.logical_or(a, b)
        ops = {"+": np.add, "-": np.subtract, "*": np.multiply, "/": np.divide, "%": np.mod, "**": np.power,
               "==": np.equal, "!=": np.not_equal, "<": np.less, "<=": np.less_equal, ">": np.greater,
               ">=": np.greater_equal}
        r = ops[op](a, b)
        return r.item() if isinstance(r, np.ndarray) and r.ndim == 0 else r
    if k == "index":
        base = evaluate(e[1], env)
        return base  # fields are per-cell values already (vectorised loops)
    if k == "member":
        v = evaluate(e[1], env)
        return np.asarray(v)[..., "xyz".index(e[2])]
    if k == "call":
        args = [evaluate(a, env) for kw, a in e[2]]
        fn = e[1]
        math1 = {"sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin, "acos": np.arccos,
                 "atan": np.arctan, "sqrt": np.sqrt, "exp": np.exp, "log": np.log, "log10": np.log10,
                 "abs": np.abs, "floor": np.floor, "ceil": np.ceil}
        if fn in math1:
            return math1[fn](args[0])
        if fn in ("min", "max", "pow", "atan2"):
            return {"min": np.minimum, "max": np.maximum, "pow": np.power, "atan2": np.arctan2}[fn](*args)
        if fn in ("vec2", "vec3", "vector"):
            return _vec(*(list(args) + [0.0] * (3 - len(args)) if fn == "vec2" else args))
        if fn == "distance":
            return np.sqrt(np.sum((np.asarray(args[0]) - np.asarray(args[1])) ** 2, -1))
        if fn == "length":
            return np.sqrt(np.sum(np.asarray(args[0]) ** 2, -1))
        if fn == "dot":
            return np.sum(np.asarray(args[0]) * np.asarray(args[1]), -1)
        if fn == "cell_position":
            if env.cell is None:
                raise ParseError("cell_position() outside a per-cell loop")
            return env.cell
        if fn in env.names and callable(env.names[fn]):
            return env.names[fn](*args)
        raise ParseError("unknown function %r" % fn)
    raise ParseError("cannot evaluate %r" % (k,))


# ---------------------------------------------------------------- scenario

# Lattice-Boltzmann kernels a `run` statement may name.
STEP_KERNELS = re.compile(r"^lbm_")
INDICATORS = ("compute_vorticity", "compute_q_criterion")


def _kw(args, env):
    return {kw: evaluate(a, env) for kw, a in args if kw}


def _period(cond):
    """N of a `timestep % N == 0` condition, else None."""
    if cond[0] == "bin" and cond[1] == "==" and cond[3] == ("num", 0):
        a = cond[2]
        if a[0] == "bin" and a[1] == "%" and a[2] == ("name", "timestep") and a[3][0] == "num":
            return int(a[3][1])
    return None


def _flag_rule(loop, fields):
    """(indicator field, refine threshold, coarsen threshold) of a per-cell loop
    `if f(X[i]) > A { refine_flag[i] = 1 } else if f(X[i]) < B { refine_flag[i] = -1 } ...`."""
    rule = {"field": None, "refine": None, "coarsen": None}

    def walk(stmts):
        for st in stmts:
            if st[0] != "if":
                continue
            cond = st[1]
            if cond[0] == "bin" and cond[1] in (">", ">=", "<", "<=") and cond[3][0] == "num":
                lhs = cond[2]
                while lhs[0] == "call":
                    lhs = lhs[2][0][1]
                if lhs[0] == "index":
                    lhs = lhs[1]
                if lhs[0] == "name" and lhs[1] in fields:
                    for s2 in st[2]:
                        if s2[0] == "assign" and s2[1] == "refine_flag" and s2[4][0] in ("num", "un"):
                            v = evaluate(s2[4], Env())
                            if v > 0 and cond[1] in (">", ">="):
                                rule["field"], rule["refine"] = lhs[1], float(cond[3][1])
                            elif v < 0 and cond[1] in ("<", "<="):
                                rule["field"], rule["coarsen"] = lhs[1], float(cond[3][1])
            walk(st[2])
            walk(st[3])

    walk(loop[4])
    return rule if rule["field"] else None


class Scenario:
    """A parsed script bound to case parameters (the benchmark cases' sizes when the
    script does not set them)."""

    def __init__(self, tree, ext=None, max_level=None, tau=None, regrid_every=None, base_dir=".", mask_level=None):
        self.tree = tree
        self.base_dir = base_dir
        self.solids = []  # placed geometries other than the case sphere: dicts of GeometryDescriptor fields
        self.fields = dict(tree["fields"])
        imports = " ".join(tree["imports"]).lower()
        self.lattice = "D3Q19"
        self.note = "D2Q9 import run as the 3-D D3Q19 case" if "d2q9" in imports else ""
        self.runs = []
        self.steps_per_iter = 0
        self.sphere = None
        self.lid = None
        self.inlet = None
        self.outlet = False
        self.rule = None
        self.regrid_every = None
        self.periodic_actions = []   # (period or 1, statement)
        self.init_u = (0.0, 0.0, 0.0)
        self._analyse()
        channel = self.inlet is not None or self.sphere is not None
        self.kind = "channel" if channel else "cavity"
        self.ext = tuple(ext) if ext else ((16, 8, 8) if channel else (4, 4, 4))
        self.max_level = max_level if max_level is not None else (3 if channel else 2)
        self.tau = tau if tau is not None else 0.56
        if regrid_every:
            self.regrid_every = regrid_every
        self.mask_level = mask_level if mask_level is not None else min(self.max_level, 2)

    def _analyse(self):
        env = Env({"timestep": 0, "num_cells": 0})
        blocks = self.tree["blocks"]
        for st in blocks.get("initial_condition", []):
            self._initial(st, env)
        for st in blocks.get("time_loop", []):
            self._loop_statement(st, env, period=None)

    def _initial(self, st, env):
        if st[0] == "place":
            self._place(st[1], env)
        elif st[0] == "for":
            for s2 in st[4]:
                if s2[0] == "assign" and s2[1] == "velocity":
                    try:
                        v = np.asarray(evaluate(s2[4], env), float).reshape(-1)
                        self.init_u = tuple(float(x) for x in (list(v) + [0, 0, 0])[:3])
                    except ParseError:
                        pass

    def _place(self, args, env):
        """place_geometry(NAME) or place_geometry(type=..., ...): the first unscaled sphere becomes the
        case's sphere; other spheres, boxes, cylinders and STL meshes become solid-mask geometry."""
        if len(args) == 1 and args[0][0] is None and args[0][1][0] == "name":  # place_geometry(NAME)
            g = self.tree["geometries"].get(args[0][1][1])
            if g is None:
                raise ParseError("place_geometry: unknown geometry %r" % args[0][1][1])
            kw = {k: (evaluate(v, env) if isinstance(v, tuple) else v) for k, v in g.items()}
        else:
            kw = _kw(args, env)
        kind = str(kw.get("type", "")).lower()
        vec = lambda v, d: tuple(float(x) for x in np.asarray(v if v is not None else d, float).reshape(-1)[:3])
        t = vec(kw.get("translate", kw.get("center")), (0.0, 0.0, 0.0))
        scale = vec(kw.get("scale"), (1.0, 1.0, 1.0))
        if kind == "sphere" and self.sphere is None and scale == (1.0, 1.0, 1.0) and not self.solids:
            self.sphere = (t, float(kw["radius"]))
            return
        if kind not in ("sphere", "box", "cylinder", "stl"):
            raise ParseError("place_geometry: type %r is not placed by this build" % kind)
        if kind == "stl" and not kw.get("source"):
            raise ParseError("place_geometry: an stl geometry needs a source file")
        self.solids.append({"type": kind, "translate": t, "scale": scale, "source": kw.get("source"),
                            **{k: float(kw.get(k, 1.0)) for k in ("radius", "height", "width", "length")}})

    def solid_geometries(self):
        """(GeometryDesc, triangles or None) of the solids in voxel units of the mask level:
        translate and scale times 2^mask_level (script coordinates are level-0 sites)."""
        from . import geometry as G
        s = float(1 << self.mask_level)
        out = []
        for g in self.solids:
            kind = {"sphere": G.SPHERE, "box": G.BOX, "cylinder": G.CYLINDER, "stl": G.STL}[g["type"]]
            d = G.make(kind, translate=[v * s for v in g["translate"]], scale=[v * s for v in g["scale"]],
                       radius=g["radius"], height=g["height"], width=g["width"], length=g["length"])
            tris = G.load_stl(os.path.join(self.base_dir, g["source"])) if kind == G.STL else None
            out.append((d, tris))
        return out

    def _loop_statement(self, st, env, period):
        k = st[0]
        if k == "run":
            name, kw = st[1], _kw(st[2], env)
            self.runs.append(name)
            if STEP_KERNELS.match(name):
                self.steps_per_iter = 1  # the lbm_* kernels of one iteration are one fused step
            elif name.startswith("apply_"):
                if "lid" in name:
                    v = kw.get("velocity_lid", 0.05)
                    self.lid = float(np.asarray(v).reshape(-1)[0])
                elif "inlet" in name:
                    v = np.asarray(kw.get("velocity_inlet", (0.04, 0.0, 0.0)), float).reshape(-1)
                    self.inlet = tuple(float(x) for x in (list(v) + [0, 0])[:3])
                elif "outlet" in name:
                    self.outlet = True
            elif name in INDICATORS:
                pass
            else:
                raise ParseError("line %d: kernel %r has no GB300 implementation" % (st[3], name))
        elif k == "for":
            r = _flag_rule(st, self.fields)
            if r:
                self.rule = r
        elif k == "if":
            p = _period(st[1])
            for s2 in st[2]:
                if s2[0] == "adapt" and p:
                    self.regrid_every = p
                elif s2[0] in ("print", "write"):
                    self.periodic_actions.append((p or 1, s2))
        elif k == "adapt":
            self.regrid_every = 1
        elif k in ("print", "write"):
            self.periodic_actions.append((1, st))

    def case(self):
        from .lbm import cavity, sphere_channel
        nx, ny, nz = (8 * e for e in self.ext)
        if self.kind == "cavity":
            c = cavity(nx, self.max_level, u_lid=self.lid if self.lid is not None else 0.05, tau=self.tau)
            c.ext[:] = list(self.ext)
        else:
            centre, radius = self.sphere if self.sphere else ((nx / 4.0, ny / 2.0, nz / 2.0), nx / 16.0)
            u = self.inlet if self.inlet else (0.04, 0.0, 0.0)
            c = sphere_channel(nx, ny, nz, self.max_level, radius=radius, centre=centre, u_in=u[0], tau=self.tau,
                               band=0.0)
            c.inlet_u[:] = list(u)
            c.init_u[:] = list(self.init_u) if any(self.init_u) else list(u)
            if self.sphere is None and self.solids:  # the placed geometry is the obstacle
                c.has_sphere = 0
        if self.rule:
            c.refine_frac = self.rule["refine"] if self.rule["refine"] is not None else c.refine_frac
            c.coarsen_frac = self.rule["coarsen"] if self.rule["coarsen"] is not None else c.coarsen_frac
        return c


# ---------------------------------------------------------------- runner

class Runner:
    """Executes a Scenario on one GPU: initial condition, `steps` time-loop
    iterations, final output."""

    def __init__(self, ctx, scenario, out_dir=".", log=print):
        from .lbm import Pool
        self.ctx, self.sc, self.out_dir, self.log = ctx, scenario, out_dir, log
        self.pool = Pool(ctx, [scenario.case()])
        self.timestep = 0
        self.lups = 0
        self.regrids = 0
        self.solid_cells = 0
        if scenario.solids:
            from . import geometry
            self.solid_cells = geometry.place(ctx, self.pool, 0, scenario.mask_level, scenario.solid_geometries())
            for _ in range(scenario.max_level):  # at rest only the mask band refines, as the sphere's at creation
                self.pool.regrid()
                self.regrids += 1

    def env(self):
        info = self.pool.info()
        return Env({"timestep": self.timestep, "num_cells": int(info.num_bricks) * 512, "pi": math.pi,
                    "compute_drag_force": lambda: float("nan")})

    def _brick_centres(self):
        b = self.pool.bricks()
        s = 1.0 / (1 << b["level"].astype(np.int64))
        return np.stack([(b[a].astype(np.float64) * 8 + 4.0) * s for a in ("x", "y", "z")], -1)

    def _prerefine(self, loops):
        """Per-cell loops writing refine_flag[i] = k under a condition, evaluated per brick centre;
        an adapt_mesh() that follows refines up to max(k) levels."""
        for rnd in range(self.sc.max_level):
            env = self.env()
            centres = self._brick_centres()
            env.cell = centres
            flags = np.zeros(len(centres), np.int32)
            for loop in loops:
                env.names[loop[1]] = np.arange(len(centres))
                self._run_masked(loop[4], env, np.ones(len(centres), bool), flags, rnd)
            if not flags.any():
                break
            self.pool.regrid_flags(flags)
            self.regrids += 1

    def _run_masked(self, stmts, env, mask, flags, rnd):
        for st in stmts:
            if st[0] == "decl":
                env.names[st[2]] = evaluate(st[3], env)
            elif st[0] == "if":
                c = np.asarray(evaluate(st[1], env), bool)
                c = np.broadcast_to(c, mask.shape)
                self._run_masked(st[2], env, mask & c, flags, rnd)
                self._run_masked(st[3], env, mask & ~c, flags, rnd)
            elif st[0] == "assign" and st[1] == "refine_flag":
                k = int(evaluate(st[4], env))
                flags[mask] = 1 if k > rnd else (-1 if k < 0 else 0)

    def _action(self, st, env=None):
        env = env or self.env()
        if st[0] == "print":
            self.log(_fmt(evaluate(st[1], env)))
        elif st[0] == "write":
            from . import io
            path = None
            for kw, a in st[2]:
                v = evaluate(a, env) if a[0] in ("str", "bin") else None
                if isinstance(v, str):
                    path = v
            if path is None:
                path = "snapshot_%06d" % self.timestep
            path = os.path.join(self.out_dir, path)
            if st[1] == "write_vtk":
                io.write_vtp(os.path.splitext(path)[0] + ".vtp", self.pool)
            else:
                io.save_snapshot(self.pool, os.path.splitext(path)[0] + ".npz")

    def initial(self):
        stmts = self.sc.tree["blocks"].get("initial_condition", [])
        flag_loops = [s for s in stmts if s[0] == "for" and self._writes_flags(s[4])]
        for st in stmts:
            if st[0] == "adapt" and flag_loops:
                self._prerefine(flag_loops)
            elif st[0] == "adapt":
                self.pool.regrid()
                self.regrids += 1
            elif st[0] in ("print", "write"):
                self._action(st)

    @staticmethod
    def _writes_flags(stmts):
        for st in stmts:
            if st[0] == "assign" and st[1] == "refine_flag" and st[4] != ("num", 0):
                return True
            if st[0] == "if" and (Runner._writes_flags(st[2]) or Runner._writes_flags(st[3])):
                return True
        return False

    def run(self, steps):
        sc = self.sc
        t0 = time.perf_counter()
        done = 0
        periods = [p for p in [sc.regrid_every] + [p for p, _ in sc.periodic_actions] if p]
        while done < steps:
            # advance to the next step at which something happens, in one call
            n = steps - done
            for p in periods:
                n = min(n, p - self.timestep % p)
            if sc.steps_per_iter:
                self.lups += self.pool.info().fluid_lups_per_step * n
                self.pool.step(n)
            done += n
            self.timestep += n
            if sc.regrid_every and self.timestep % sc.regrid_every == 0:
                self.pool.regrid()
                self.regrids += 1
            for p, st in sc.periodic_actions:
                if self.timestep % p == 0:
                    self._action(st)
        self.ctx.sync()
        return time.perf_counter() - t0

    def final(self):
        env = self.env()
        for st in self.sc.tree["blocks"].get("final_output", []):
            if st[0] in ("print", "write"):
                self._action(st, env)
            elif st[0] == "decl":  # e.g. `float drag = compute_drag_force()` (NaN: not provided)
                env.names[st[2]] = evaluate(st[3], env)


def main(argv=None):
    ap = argparse.ArgumentParser(description="Run a .fl simulation script on one GPU")
    ap.add_argument("script")
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--ext", type=int, nargs=3, help="level-0 bricks per axis (8 sites each)")
    ap.add_argument("--max-level", type=int)
    ap.add_argument("--tau", type=float)
    ap.add_argument("--regrid-every", type=int)
    ap.add_argument("--mask-level", type=int, help="level of the solid-mask grid of placed geometries")
    ap.add_argument("--out", default="fl_output")
    args = ap.parse_args(argv)
    from . import Context
    tree = parse(open(args.script).read())
    sc = Scenario(tree, args.ext, args.max_level, args.tau, args.regrid_every,
                  base_dir=os.path.dirname(os.path.abspath(args.script)), mask_level=args.mask_level)
    ctx = Context(0)
    r = Runner(ctx, sc, args.out)
    r.initial()
    secs = r.run(args.steps)
    r.final()
    info = r.pool.info()
    res = {"script": os.path.basename(args.script), "kind": sc.kind, "lattice": sc.lattice, "note": sc.note,
           "steps": args.steps, "regrids": r.regrids, "solid_cells": r.solid_cells, "bricks": int(info.num_bricks), "seconds": secs,
           "mlups": r.lups / secs / 1e6 if secs > 0 else None, "kernels": sc.runs}
    print(json.dumps(res))
    return res


if __name__ == "__main__":
    main()
