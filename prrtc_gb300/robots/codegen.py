"""Robot-model compiler: JSON collision models -> C tables + CUDA checkers.

Input: ``prrtc_gb300/robots/<robot>.json`` (written by ``extract.py``).
Output, for each robot:

* ``csrc/robots/<robot>_model.h``: the model as plain-C tables
  (``prrtc_joint_def`` ... from ``model_types.h``), read by the CPU oracle and
  by host code;
* ``csrc/robots/<robot>_fkcc.cuh``: a straight-line CUDA forward-kinematics
  and collision-check routine for one configuration per thread.  Joint
  transforms are folded at generation time (zero and unit entries of the
  fixed transforms vanish), every frame lives in registers, and the checker
  visits the model's groups in the reference's order.  The per-leaf work runs
  in three small shared routines supplied by the caller (``Ctx``), so code
  size stays proportional to the number of groups, not of sphere pairs:

  - ``ctx.env_hit(x, y, z, r)``: sphere against every obstacle;
  - ``ctx.env_leaves(T, leaves, n)``: leaf spheres given in frame T;
  - ``ctx.self_pairs(Tab, pairs, n)``: sphere pairs (a in frame A, b in
    frame B) given the relative transform Tab = inv(T_A) T_B;
  - ``ctx.pair_hit(dx, dy, dz, ra + rb)``: gate pair overlap test;
  - ``ctx.stop()``: cooperative early exit (another lane already failed).

Usage: ``python -m prrtc_gb300.robots.codegen`` (no reference checkout needed).
"""
from __future__ import annotations

import json
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "csrc" / "robots"
ROBOTS = ("sphere", "panda", "fetch", "baxter")
INLINE_LEAVES = 6   # leaf blocks up to this size are emitted as straight-line tests
# Robots whose checker is emitted in table form: every frame computed first,
# then one loop over the group schedule (run_schedule in device_common.cuh).
# Baxter's 388 groups as straight-line code overflow the instruction cache
# (its planner kernel stalled on instruction fetch 33 times per issue).
TABLE_ROBOTS = ("panda", "fetch", "baxter")
# Robots that also get the straight-line form, as fkcc_validate: Panda's
# stand-alone checker runs 6 % faster with it than with the table form (2^20
# random configurations, tabletop scene: 1.24 vs 1.32 ms).  Fetch's runs 2 %
# faster in table form at 64 registers (mixed scene: 5.28 vs 5.38 ms) and
# Baxter's straight-line form does not fit the instruction cache, so both
# use the table form for single configurations too.
INLINE_VALIDATE = ("sphere", "panda")


def load_model(robot: str) -> dict:
    return json.loads((HERE / f"{robot}.json").read_text())


def _lit(x: float) -> str:
    x = float(x)
    if x == int(x) and abs(x) < 1e6:
        return f"{x:.1f}f"
    return f"{x!r}f"


# ------------------------------------------------------------------ C tables

def emit_c_tables(m: dict) -> str:
    R = m["robot"].capitalize()
    out = []
    w = out.append
    w(f"// pRRTC {m['robot']} collision model as plain-C tables.  Generated by")
    w("// prrtc_gb300/robots/codegen.py from the fitted model; do not edit.")
    w(f"// Max |sphere centre - reference float64 FK|: {m['max_err']:.3e} m")
    w("#pragma once")
    w('#include "model_types.h"')
    w("")
    ne, ns = len(m["env_groups"]), len(m["self_groups"])
    nl = sum(len(g["leaves"]) for g in m["env_groups"])
    npairs = sum(len(g["pairs"]) for g in m["self_groups"])
    w("enum {")
    w(f"    k{R}Dof = {m['dof']},")
    w(f"    k{R}NumJoints = {len(m['joints'])},")
    w(f"    k{R}NumSpheres = {len(m['spheres'])},")
    w(f"    k{R}NumEnvGroups = {ne},")
    w(f"    k{R}NumEnvLeaves = {nl},")
    w(f"    k{R}NumSelfGroups = {ns},")
    w(f"    k{R}NumSelfPairs = {npairs},")
    w(f"    k{R}NumSchedule = {len(m['schedule'])},")
    w("};")
    w("")
    w(f"static const prrtc_joint_def k{R}Joints[] = {{")
    for jt in m["joints"]:
        F = [x for row in jt["F"] for x in row]
        w("    {%d, %d, %d, {%s}}," % (jt["q"], jt["parent"], 1 if jt["type"] == "revolute" else 0,
                                     ", ".join(_lit(x) for x in F)))
    w("};")
    w(f"static const prrtc_sphere_def k{R}Spheres[] = {{")
    for s in m["spheres"]:
        w("    {%d, %s, %s, %s, %s}," % (s["frame"], *[_lit(x) for x in s["c"]], _lit(s["r"])))
    w("};")
    w(f"static const prrtc_group_def k{R}EnvGroups[] = {{")
    off = 0
    for g in m["env_groups"]:
        w("    {%d, -1, %d, %d},  /* %s */" % (g["gate"], off, len(g["leaves"]), g["label"]))
        off += len(g["leaves"])
    w("};")
    allv = [x for g in m["env_groups"] for x in g["leaves"]]
    w(f"static const short k{R}EnvLeaves[] = {{")
    for i in range(0, len(allv), 16):
        w("    " + ", ".join(str(x) for x in allv[i:i + 16]) + ",")
    w("};")
    if ns:
        w(f"static const prrtc_group_def k{R}SelfGroups[] = {{")
        off = 0
        for g in m["self_groups"]:
            w("    {%d, %d, %d, %d},  /* %s */" % (g["gate"][0], g["gate"][1], off, len(g["pairs"]), g["label"]))
            off += len(g["pairs"])
        w("};")
        allp = [p for g in m["self_groups"] for p in g["pairs"]]
        w(f"static const short k{R}SelfPairs[][2] = {{")
        for i in range(0, len(allp), 8):
            w("    " + " ".join("{%d, %d}," % tuple(p) for p in allp[i:i + 8]))
        w("};")
    else:
        w(f"static const prrtc_group_def k{R}SelfGroups[] = {{{{-1, -1, 0, 0}}}};")
        w(f"static const short k{R}SelfPairs[][2] = {{{{0, 0}}}};")
    w(f"static const prrtc_sched_def k{R}Schedule[] = {{")
    for i in range(0, len(m["schedule"]), 8):
        w("    " + " ".join("{%d, %d}," % (0 if k == "env" else 1, g) for k, g in m["schedule"][i:i + 8]))
    w("};")
    w("")
    return "\n".join(out)


# ------------------------------------------------------- symbolic scalar code

class _Code:
    """Straight-line float code with constant folding of 0 / +-1 / literals."""

    def __init__(self):
        self.lines = []
        self.n = 0

    def tmp(self, expr, prefix="v"):
        if isinstance(expr, float):
            return expr
        name = f"{prefix}{self.n}"
        self.n += 1
        self.lines.append(f"const float {name} = {expr};")
        return name

    @staticmethod
    def term(coef: float, var):
        """coef * var as (sign, text) or a folded constant."""
        if isinstance(var, float):
            return coef * var
        if coef == 0.0:
            return 0.0
        if coef == 1.0:
            return var
        if coef == -1.0:
            return f"(-{var})"
        return f"{_lit(coef)} * {var}"

    @staticmethod
    def dot(pairs, const=0.0):
        """sum(coef * var) + const; coef may be a float or a variable name,
        var may be a variable name or a float."""
        c = float(const)
        terms = []
        for a, b in pairs:
            if isinstance(a, float) and isinstance(b, float):
                c += a * b
            elif isinstance(a, float) or isinstance(b, float):
                k, v = (a, b) if isinstance(a, float) else (b, a)
                if k == 0.0:
                    continue
                terms.append(_Code.term(k, v))
            else:
                terms.append(f"{a} * {b}")
        if not terms:
            return c
        s = terms[0]
        for t in terms[1:]:
            if t.startswith("(-"):
                s = f"{s} - {t[2:-1]}"
            else:
                s = f"{s} + {t}"
        if c != 0.0:
            s = f"{s} + {_lit(c)}" if c > 0 else f"{s} - {_lit(-c)}"
        return s


def _mat_of(F):
    return [[float(F[i][k]) for k in range(4)] for i in range(3)]


class _FkGen:
    """Emits frame computations lazily, in chain order, into a _Code."""

    def __init__(self, model, code: _Code):
        self.m = model
        self.code = code
        self.frames = {-1: [[1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0]]}
        self.joint = {jt["q"]: jt for jt in model["joints"]}

    def frame(self, j):
        if j in self.frames:
            return self.frames[j]
        jt = self.joint[j]
        P = self.frame(jt["parent"])
        F = _mat_of(jt["F"])
        c = self.code
        # A = P * F   (3x4 affine composition)
        A = [[None] * 4 for _ in range(3)]
        for i in range(3):
            for k in range(3):
                A[i][k] = c.tmp(c.dot([(P[i][m], F[m][k]) for m in range(3)]), f"a{j}_")
            A[i][3] = c.tmp(c.dot([(P[i][m], F[m][3]) for m in range(3)] + [(P[i][3], 1.0)]), f"a{j}_")
        q = f"q[{j}]"
        T = [[None] * 4 for _ in range(3)]
        if jt["type"] == "revolute":
            # T = A * Rz(q): columns 0 and 1 rotate, column 2 and the origin stay
            s, co = f"s{j}", f"c{j}"
            c.lines.append(f"float {s}, {co};")
            c.lines.append(f"sincosf({q}, &{s}, &{co});")
            for i in range(3):
                T[i][0] = c.tmp(c.dot([(co, A[i][0]), (s, A[i][1])]), f"t{j}_")
                T[i][1] = c.tmp(_sub(c, c.dot([(co, A[i][1])]), c.dot([(s, A[i][0])])), f"t{j}_")
                T[i][2] = A[i][2]
                T[i][3] = A[i][3]
        else:
            # T = A * Tz(q): the origin slides along column 2
            for i in range(3):
                T[i][0], T[i][1], T[i][2] = A[i][0], A[i][1], A[i][2]
                T[i][3] = c.tmp(c.dot([(A[i][3], 1.0), (q, A[i][2])]), f"t{j}_")
        self.frames[j] = T
        return T

    def point(self, f, xyz):
        """World coordinates of a point given in frame f."""
        T = self.frame(f)
        return [self.code.tmp(self.code.dot([(T[i][k], float(xyz[k])) for k in range(3)] + [(T[i][3], 1.0)]), "p")
                for i in range(3)]

    def relative(self, fa, fb):
        """Tab = inv(T_fa) * T_fb as a 3x4 of operands."""
        c = self.code
        Ta, Tb = self.frame(fa), self.frame(fb)
        d = [c.tmp(_sub(c, Tb[i][3], Ta[i][3]), "d") for i in range(3)]
        M = [[None] * 4 for _ in range(3)]
        for i in range(3):
            for k in range(3):
                M[i][k] = c.tmp(c.dot([(Ta[m][i], Tb[m][k]) for m in range(3)]), "r")
            M[i][3] = c.tmp(c.dot([(Ta[m][i], d[m]) for m in range(3)]), "r")
        return M


def _sub(c: _Code, a, b):
    """a - b over operands/expressions (strings are wrapped)."""
    if isinstance(a, float) and isinstance(b, float):
        return a - b
    if isinstance(b, float):
        if b == 0.0:
            return a
        return f"({a}) - {_lit(b)}" if b > 0 else f"({a}) + {_lit(-b)}"
    if isinstance(a, float) and a == 0.0:
        return f"-({b})"
    return f"({a}) - ({b})"


def _frame_arg(M):
    vals = []
    for i in range(3):
        for k in range(4):
            v = M[i][k]
            vals.append(_lit(v) if isinstance(v, float) else v)
    return "Frame{{" + ", ".join(vals) + "}}"


def emit_cuda_checker(m: dict) -> str:
    name = m["robot"]
    R = name.capitalize()
    sp = m["spheres"]
    code = _Code()
    fk = _FkGen(m, code)
    body = []

    # leaf tables: env leaves grouped into same-frame blocks; self pairs into
    # same-(frame a, frame b) blocks.  Blocks keep the reference's order.
    leaf_rows, pair_rows = [], []
    env_blocks, self_blocks = {}, {}
    for gi, g in enumerate(m["env_groups"]):
        blocks = []
        for leaf in g["leaves"]:
            f = sp[leaf]["frame"]
            if not blocks or blocks[-1][0] != f:
                blocks.append([f, len(leaf_rows), 0])
            s = sp[leaf]
            leaf_rows.append((s["c"][0], s["c"][1], s["c"][2], s["r"]))
            blocks[-1][2] += 1
        env_blocks[gi] = blocks
    for gi, g in enumerate(m["self_groups"]):
        blocks = []
        for a, b in g["pairs"]:
            fa, fb = sp[a]["frame"], sp[b]["frame"]
            if not blocks or (blocks[-1][0], blocks[-1][1]) != (fa, fb):
                blocks.append([fa, fb, len(pair_rows), 0])
            pair_rows.append((sp[a]["c"], sp[a]["r"], sp[b]["c"], sp[b]["r"]))
            blocks[-1][3] += 1
        self_blocks[gi] = blocks

    def env_block_calls(gi):
        """Leaf tests of an environment group: blocks of up to INLINE_LEAVES
        spheres are tested inline (centres folded at generation time), larger
        ones through ctx.env_leaves over the leaf table."""
        calls = []
        for f, first, n in env_blocks[gi]:
            T = fk.frame(f)
            if n <= INLINE_LEAVES:
                for k in range(first, first + n):
                    x, y, z, r = leaf_rows[k]
                    p = fk.point(f, (x, y, z))
                    calls.append(f"ctx.env_hit({_op(p[0])}, {_op(p[1])}, {_op(p[2])}, {_lit(r)})")
            else:
                calls.append(f"ctx.env_leaves({_frame_arg(T)}, k{R}Leaf + {first}, {n})")
        return calls

    table = name in TABLE_ROBOTS
    inline = not table or name in INLINE_VALIDATE
    # the gate spheres (environment groups' bounding spheres and self groups'
    # bounding pairs), each once, in order of first use
    gate_ids = {}
    for g in m["env_groups"]:
        if g["gate"] >= 0:
            gate_ids.setdefault(g["gate"], len(gate_ids))
    for g in m["self_groups"]:
        for sidx in g["gate"]:
            gate_ids.setdefault(sidx, len(gate_ids))
    tcode = None
    if table:
        # every frame, in chain order, into F[q + 1]; then the schedule loop
        nj = len(m["joints"])
        frames = [fk.frame(jt["q"]) for jt in m["joints"]]
        code.lines.append(f"FrameStore<Ctx, {nj + 1}> F(ctx);")
        code.lines.append("F.set(0, Frame{{1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f}});")
        for jt, T in zip(m["joints"], frames):
            code.lines.append(f"F.set({jt['q'] + 1}, {_frame_arg(T)});")
        # gate centres in world coordinates, from the frames still in registers
        # (the schedule walk then reads 16 bytes per gate test, not a frame)
        fexpr = {-1: "world_frame()"} | {jt["q"]: _frame_arg(T) for jt, T in zip(m["joints"], frames)}
        code.lines.append(f"float4 G[{max(1, len(gate_ids))}];")
        for sidx, gid in gate_ids.items():
            code.lines.append(f"G[{gid}] = gate_centre({fexpr[sp[sidx]['frame']]}, k{R}Gate[{gid}]);")
        code.lines.append(f"return run_schedule(F.view(), G, k{R}Sched, {len(m['schedule'])}, k{R}EnvGroup, k{R}LeafBlock, k{R}Leaf, "
                          f"k{R}SelfGroup, k{R}PairBlock, k{R}Pair, ctx);")
        tcode = code
        code = _Code()              # the straight-line form, if any, goes to its own code
        fk = _FkGen(m, code)
    for kind, gi in (m["schedule"] if inline else []):
        if kind == "env":
            g = m["env_groups"][gi]
            code.lines.append(f"// environment group {gi}: {g['label']}")
            for f, _, _ in env_blocks[gi]:       # frames are shared: compute outside the if
                fk.frame(f)
            if g["gate"] >= 0:
                s = sp[g["gate"]]
                x, y, z = fk.point(s["frame"], s["c"])
                code.lines.append(f"if (ctx.env_hit({_op(x)}, {_op(y)}, {_op(z)}, {_lit(s['r'])})) {{")
                for call in env_block_calls(gi):
                    code.lines.append(f"    if ({call}) return false;")
                code.lines.append("}")
            else:
                for call in env_block_calls(gi):
                    code.lines.append(f"if ({call}) return false;")
        else:
            g = m["self_groups"][gi]
            code.lines.append(f"// self group {gi}: {g['label']}")
            a, b = g["gate"]
            sa, sb = sp[a], sp[b]
            pa = fk.point(sa["frame"], sa["c"])
            pb = fk.point(sb["frame"], sb["c"])
            for fa, fb, _, _ in self_blocks[gi]:  # frames are shared: compute outside the if
                fk.frame(fa)
                fk.frame(fb)
            dx, dy, dz = (code.tmp(_sub(code, pa[i], pb[i]), "g") for i in range(3))
            code.lines.append(f"if (ctx.pair_hit({_op(dx)}, {_op(dy)}, {_op(dz)}, {_lit(sa['r'])} + {_lit(sb['r'])})) {{")
            for fa, fb, first, n in self_blocks[gi]:
                M = fk.relative(fa, fb)
                code.lines.append(f"    if (ctx.self_pairs({_frame_arg(M)}, k{R}Pair + {first}, {n})) return false;")
            code.lines.append("}")
        code.lines.append("if (ctx.stop()) return true;")
    if inline:
        code.lines.append("return true;")

    # fk_spheres: every sphere's world centre (not on the validation hot path)
    code2 = _Code()
    fk2 = _FkGen(m, code2)
    for i, s in enumerate(sp):
        x, y, z = fk2.point(s["frame"], s["c"])
        code2.lines.append(f"out[{i}] = make_float4({_op(x)}, {_op(y)}, {_op(z)}, {_lit(s['r'])});")

    out = []
    w = out.append
    w(f"// Straight-line CUDA collision checker for pRRTC's {name} model.  Generated by")
    w("// prrtc_gb300/robots/codegen.py from the fitted model; do not edit.")
    w("// Semantics follow the reference checker fkcc<Robot> (src/planning/utils.cuh):")
    w("// a leaf counts only when its group's gate (bounding sphere or bounding pair)")
    w("// is hit; a config is free when no counted leaf is hit.")
    w("#pragma once")
    w("")
    w(f"namespace prrtc {{ namespace gen_{name} {{")
    w("")
    w(f"constexpr int kDof = {m['dof']};")
    w(f"constexpr int kFrames = {len(m['joints']) + 1};   // the world and one frame per joint")
    w(f"constexpr int kNumSpheres = {len(sp)};")
    w(f"constexpr int kNumLeaves = {max(1, len(leaf_rows))};")
    w(f"constexpr int kNumPairs = {max(1, len(pair_rows))};")
    w("// canonical algorithmic FLOPs of one forward kinematics: 2 * (12 * dof + 9 * spheres)")
    w(f"constexpr unsigned kFkFlops = {2 * (12 * m['dof'] + 9 * len(sp))}u;")
    w("")
    w("// leaf spheres in their frame: (x, y, z, r)")
    w(f"__device__ const float4 k{R}Leaf[kNumLeaves] = {{")
    for r in leaf_rows or [(0.0, 0.0, 0.0, 0.0)]:
        w("    {%s}," % ", ".join(_lit(v) for v in r))
    w("};")
    w("// sphere pairs: a = (x, y, z, r) in frame A, b = (x, y, z, r) in frame B")
    w(f"__device__ const LeafPair k{R}Pair[kNumPairs] = {{")
    for ca, ra, cb, rb in pair_rows or [([0, 0, 0], 0.0, [0, 0, 0], 0.0)]:
        w("    {{%s, %s, %s, %s}, {%s, %s, %s, %s}}," % (*[_lit(v) for v in ca], _lit(ra), *[_lit(v) for v in cb], _lit(rb)))
    w("};")
    if table:
        w("// the schedule in table form (run_schedule)")
        w(f"__device__ const GenSched k{R}Sched[{len(m['schedule'])}] = {{")
        for kind, gi in m["schedule"]:
            w(f"    {{{0 if kind == 'env' else 1}, {gi}}},")
        w("};")
        lblocks, eg_rows = [], []
        for gi, g in enumerate(m["env_groups"]):
            first = len(lblocks)
            for f, fl, n in env_blocks[gi]:
                lblocks.append((f, fl, n))
            eg_rows.append((gate_ids[g["gate"]] if g["gate"] >= 0 else -1, first, len(lblocks) - first))
        w("// gate spheres (x, y, z, r) in their frames; gate_centre() puts them in the world")
        w(f"__device__ const float4 k{R}Gate[{max(1, len(gate_ids))}] = {{")
        for sidx in gate_ids or [None]:
            c = sp[sidx] if sidx is not None else {"c": [0.0, 0.0, 0.0], "r": 0.0}
            w("    {%s, %s, %s, %s}," % (*[_lit(v) for v in c["c"]], _lit(c["r"])))
        w("};")
        w(f"__device__ const GenEnvGroup k{R}EnvGroup[{max(1, len(eg_rows))}] = {{")
        for gid, first, nb in eg_rows or [(-1, 0, 0)]:
            w(f"    {{{gid}, {first}, {nb}, 0}},")
        w("};")
        w(f"__device__ const GenLeafBlock k{R}LeafBlock[{max(1, len(lblocks))}] = {{")
        for f, fl, n in lblocks or [(-1, 0, 0)]:
            w(f"    {{{f}, {fl}, {n}, 0}},")
        w("};")
        pblocks, sg_rows = [], []
        for gi, g in enumerate(m["self_groups"]):
            first = len(pblocks)
            for fa, fb, pf, n in self_blocks[gi]:
                pblocks.append((fa, fb, pf, n))
            a, b = g["gate"]
            sg_rows.append((gate_ids[a], gate_ids[b], first, len(pblocks) - first))
        w(f"__device__ const GenSelfGroup k{R}SelfGroup[{max(1, len(sg_rows))}] = {{")
        for ga, gb, first, nb in sg_rows or [(0, 0, 0, 0)]:
            w(f"    {{{ga}, {gb}, {first}, {nb}}},")
        w("};")
        w(f"__device__ const GenPairBlock k{R}PairBlock[{max(1, len(pblocks))}] = {{")
        for fa, fb, pf, n in pblocks or [(-1, -1, 0, 0)]:
            w(f"    {{{fa}, {fb}, {pf}, {n}}},")
        w("};")
    w("")
    w("// Returns true when configuration q is collision-free.")
    w("template <class Ctx>")
    w("__device__ __forceinline__ bool fkcc(const float *__restrict__ q, Ctx &ctx)")
    w("{")
    for line in (tcode if table else code).lines:
        w("    " + line)
    w("}")
    w("")
    w("// The same verdicts for the stand-alone checker of single configurations.")
    w("template <class Ctx>")
    w("__device__ __forceinline__ bool fkcc_validate(const float *__restrict__ q, Ctx &ctx)")
    w("{")
    if table and inline:
        for line in code.lines:
            w("    " + line)
    else:
        w("    return fkcc(q, ctx);")
    w("}")
    w("")
    w("// World centre and radius of every model sphere (model sphere order).")
    w("__device__ __forceinline__ void fk_spheres(const float *__restrict__ q, float4 *__restrict__ out)")
    w("{")
    for line in code2.lines:
        w("    " + line)
    w("}")
    w("")
    w(f"}} }}  // namespace prrtc::gen_{name}")
    w("")
    return "\n".join(out)


def _op(v):
    return _lit(v) if isinstance(v, float) else v


def write_all():
    for r in ROBOTS:
        m = load_model(r)
        (CSRC / f"{r}_model.h").write_text(emit_c_tables(m))
        (CSRC / f"{r}_fkcc.cuh").write_text(emit_cuda_checker(m))


def check_up_to_date() -> list:
    """Names of generated files that differ from what the JSON models give."""
    stale = []
    for r in ROBOTS:
        m = load_model(r)
        for path, text in ((CSRC / f"{r}_model.h", emit_c_tables(m)), (CSRC / f"{r}_fkcc.cuh", emit_cuda_checker(m))):
            if not path.exists() or path.read_text() != text:
                stale.append(path.name)
    return stale


if __name__ == "__main__":
    write_all()
