"""Reader for pRRTC's generated per-robot collision checkers.

pRRTC ships its robot models only as generated CUDA: one straight-line
``fkcc<Robot>`` function per robot in ``src/planning/utils.cuh``
(Panda ``utils.cuh:336-5270``, Fetch ``:5272-19882``, Baxter
``:19884-33131``; the toy Sphere robot ``:330-334`` has no FK).  Each body is

* single-assignment scalar statements ``float|auto NAME = expr;`` whose
  expressions are one of ``a*b``, ``a+b``, ``a-b``, ``-a``, ``sin(a)``,
  ``cos(a)`` or ``q[i]`` over names and decimal literals, and
* nested ``if (test(...)) { ... return false; }`` blocks, where ``test`` is
  ``sphere_environment_in_collision(environment, x, y, z, r)`` or
  ``sphere_sphere_self_collision(ax, ay, az, ar, bx, by, bz, br)``.

This module parses such a body into a value DAG plus a decision tree and
evaluates the DAG in float64 for a batch of joint configurations.  It is
used at model-build time (``extract.py`` derives the kinematic model that
the CUDA kernels compile in) and by the test-suite as the float64 forward
kinematics of the reference model.  Nothing at library run time imports it.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

# (robot name, C++ specialisation tag) in the order they appear in utils.cuh
ROBOT_TAGS = {
    "sphere": "ppln::robots::Sphere",
    "panda": "ppln::robots::Panda",
    "fetch": "ppln::robots::Fetch",
    "baxter": "ppln::robots::Baxter",
}

_NUM = r"-?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"
_NAME = r"[A-Za-z_][A-Za-z0-9_]*"
_ASSIGN = re.compile(rf"^(?:float|auto|double|const float|const auto)\s+({_NAME})\s*=\s*(.+)$")
_BIN = re.compile(rf"^({_NAME}|{_NUM})\s*([*+\-/])\s*({_NAME}|{_NUM})$")
_UN_NEG = re.compile(rf"^-\s*({_NAME})$")
_FUNC = re.compile(rf"^(sin|cos|sqrt)\s*\(\s*({_NAME}|{_NUM})\s*\)$")
_INPUT = re.compile(r"^q\s*\[\s*(\d+)\s*\]$")
_ATOM = re.compile(rf"^({_NAME}|{_NUM})$")
_IF = re.compile(r"^if\s*\(\s*(sphere_environment_in_collision|sphere_sphere_self_collision)\s*\((.*)\)\s*\)$")


@dataclass
class Test:
    """One guarded primitive test of the generated checker.

    ``kind`` is ``"env"`` (sphere against every obstacle) or ``"self"``
    (sphere against sphere).  ``args`` are operands: a name of the DAG or a
    float literal; 4 for env tests, 8 for self tests.  ``children`` are the
    tests nested inside the block; ``returns`` is True when the block body
    contains ``return false`` (collision) directly.
    """

    kind: str
    args: list
    children: list = field(default_factory=list)
    returns: bool = False
    label: str = ""


@dataclass
class Program:
    robot: str
    defs: list            # (name, op, a, b) in program order
    tests: list           # top-level Test blocks, in program order
    inputs: dict          # name -> config index

    @property
    def dof(self) -> int:
        return max(self.inputs.values()) + 1 if self.inputs else 3


def _strip_comments(text: str) -> tuple[str, list]:
    """Remove comments, keeping ``/*label*/`` markers found inside ``if (``."""
    text = re.sub(r"//[^\n]*", "", text)
    labels = []

    def keep(m):
        labels.append(m.group(1).strip())
        return f" @@L{len(labels) - 1}@@ "

    text = re.sub(r"/\*(.*?)\*/", keep, text, flags=re.S)
    return text, labels


def _body_of(source: str, tag: str) -> str:
    head = re.search(r"template\s*<>\s*__device__\s+__forceinline__\s+bool\s+fkcc<" + re.escape(tag) + r">\s*\([^)]*\)\s*\{",
                     source)
    if head is None:
        raise ValueError(f"fkcc<{tag}> not found")
    i = head.end()
    depth = 1
    j = i
    while depth:
        c = source[j]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        j += 1
    return source[i:j - 1]


def _operand(tok: str):
    tok = tok.strip()
    if re.fullmatch(_NUM, tok):
        return float(tok)
    if re.fullmatch(_NAME, tok):
        return tok
    raise ValueError(f"bad operand {tok!r}")


def parse_program(source: str, robot: str) -> Program:
    body, labels = _strip_comments(_body_of(source, ROBOT_TAGS[robot]))
    # statements end at ';' ; blocks delimit with '{' '}'
    toks = re.findall(r"[^;{}]+|[;{}]", body)
    defs, inputs = [], {}
    root: list = []
    stack: list = [root]
    stack_tests: list = [Test("root", [])]
    pending_if = None
    for raw in toks:
        t = " ".join(raw.split())
        if not t:
            continue
        if t == "{":
            if pending_if is None:
                raise ValueError("unexpected block")
            stack.append(pending_if.children)
            stack_tests.append(pending_if)
            pending_if = None
            continue
        if t == "}":
            stack.pop()
            stack_tests.pop()
            continue
        if t == ";":
            continue
        lab = ""
        m_lab = re.search(r"@@L(\d+)@@", t)
        if m_lab:
            lab = labels[int(m_lab.group(1))]
            t = re.sub(r"\s*@@L\d+@@\s*", " ", t).strip()
            t = t.replace("( ", "(").replace(" )", ")")
        if t.startswith("if"):
            m = _IF.match(t.replace("( ", "(").replace(" (", "("))
            if m is None:
                m = _IF.match(re.sub(r"\s*\(\s*", "(", t))
            if m is None:
                raise ValueError(f"unparsed if: {t!r}")
            fn, argstr = m.group(1), m.group(2)
            args = [a.strip() for a in argstr.split(",")]
            if fn == "sphere_environment_in_collision":
                if args[0] != "environment":
                    raise ValueError(t)
                test = Test("env", [_operand(a) for a in args[1:]], label=lab)
            else:
                test = Test("self", [_operand(a) for a in args], label=lab)
            if len(test.args) != (4 if test.kind == "env" else 8):
                raise ValueError(t)
            stack[-1].append(test)
            pending_if = test
            continue
        if t == "return false":
            stack_tests[-1].returns = True
            continue
        if t == "return true":
            continue
        if t.startswith("return"):
            # the toy Sphere robot: `return not sphere_environment_in_collision(...)`
            raise ValueError(f"unsupported return: {t!r}")
        m = _ASSIGN.match(t)
        if m is None:
            raise ValueError(f"unparsed statement: {t!r}")
        name, expr = m.group(1), m.group(2).strip()
        if (mi := _INPUT.match(expr)):
            inputs[name] = int(mi.group(1))
            defs.append((name, "input", int(mi.group(1)), None))
        elif (mb := _BIN.match(expr)):
            op = {"*": "mul", "+": "add", "-": "sub", "/": "div"}[mb.group(2)]
            defs.append((name, op, _operand(mb.group(1)), _operand(mb.group(3))))
        elif (mn := _UN_NEG.match(expr)):
            defs.append((name, "neg", _operand(mn.group(1)), None))
        elif (mf := _FUNC.match(expr)):
            defs.append((name, mf.group(1), _operand(mf.group(2)), None))
        elif (ma := _ATOM.match(expr)):
            defs.append((name, "copy", _operand(ma.group(1)), None))
        else:
            raise ValueError(f"unparsed expression: {expr!r}")
    return Program(robot, defs, root, inputs)


def load_program(reference_root: str | Path, robot: str) -> Program:
    src = (Path(reference_root) / "src/planning/utils.cuh").read_text()
    return parse_program(src, robot)


def evaluate(prog: Program, q: np.ndarray) -> dict:
    """Evaluate every DAG value in float64 for a batch ``q`` of shape (N, D)."""
    q = np.asarray(q, dtype=np.float64)
    vals: dict = {}

    def get(a):
        return a if isinstance(a, float) else vals[a]

    for name, op, a, b in prog.defs:
        if op == "input":
            vals[name] = q[:, a]
        elif op == "mul":
            vals[name] = get(a) * get(b)
        elif op == "add":
            vals[name] = get(a) + get(b)
        elif op == "sub":
            vals[name] = get(a) - get(b)
        elif op == "div":
            vals[name] = get(a) / get(b)
        elif op == "neg":
            vals[name] = -get(a)
        elif op == "sin":
            vals[name] = np.sin(get(a))
        elif op == "cos":
            vals[name] = np.cos(get(a))
        elif op == "sqrt":
            vals[name] = np.sqrt(get(a))
        elif op == "copy":
            vals[name] = get(a)
        else:
            raise ValueError(op)
    return vals


def operand_value(vals: dict, a, n: int) -> np.ndarray:
    if isinstance(a, float):
        return np.full(n, a)
    return np.broadcast_to(vals[a], (n,)).astype(np.float64)


def dependencies(prog: Program) -> dict:
    """For every DAG name, the set of config indices it depends on."""
    dep: dict = {}
    for name, op, a, b in prog.defs:
        if op == "input":
            dep[name] = frozenset([a])
            continue
        s = frozenset()
        for x in (a, b):
            if isinstance(x, str):
                s = s | dep[x]
        dep[name] = s
    return dep


def iter_tests(tests, parent=None):
    for t in tests:
        yield t, parent
        yield from iter_tests(t.children, t)
