"""A small Quil front end for the pure-state path.

It parses the subset of Quil the statevector path executes: DECLARE,
standard and DEFGATE'd gate applications (matrix and PERMUTATION forms, with
parameters), the DAGGER / CONTROLLED modifiers, MEASURE (with or without a
memory reference), RESET, NOP, HALT, PRAGMA and comments.  The reference
delegates parsing to cl-quil (``quil:parse-quil``); this front end only has
to produce the instruction stream that src/transition.lisp executes.
"""
from __future__ import annotations

import ast
import math
import re
from dataclasses import dataclass, field

import numpy as np

from .gates import STANDARD_GATES, controlled, dagger, gate_matrix


@dataclass
class GateApp:
    name: str
    matrix: np.ndarray
    args: list          # Quil argument order
    kind: str = "dense"  # "dense" or "perm"
    perm: list | None = None

    @property
    def qubits(self):
        """nat-tuple order (src/utilities.lisp:43-51)."""
        return list(reversed(self.args))


@dataclass
class Measure:
    qubit: int
    mref: tuple | None  # (name, index)


@dataclass
class MeasureAll:
    """The measure-chain pseudo-instruction (src/compile-gate.lisp:538-599)."""
    storage: list       # [(qubit, (name, index)) ...]


@dataclass
class Reset:
    pass


@dataclass
class Program:
    instructions: list = field(default_factory=list)
    memory: dict = field(default_factory=dict)  # name -> length

    def qubits_needed(self) -> int:
        m = -1
        for ins in self.instructions:
            if isinstance(ins, GateApp):
                m = max([m] + ins.args)
            elif isinstance(ins, Measure):
                m = max(m, ins.qubit)
        return m + 1


_ALLOWED_FUNCS = {"sin": math.sin, "cos": math.cos, "sqrt": math.sqrt, "exp": np.exp,
                  "cis": lambda x: complex(math.cos(x), math.sin(x))}


def eval_expr(text: str, env: dict | None = None):
    """Evaluate a Quil arithmetic expression (pi, i, %params, + - * / ^)."""
    env = dict(env or {})
    src = text.strip().replace("^", "**")
    src = re.sub(r"%([A-Za-z_][A-Za-z0-9_]*)", r"__p_\1", src)
    tree = ast.parse(src, mode="eval")

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return node.value
        if isinstance(node, ast.Name):
            if node.id == "pi":
                return math.pi
            if node.id == "i":
                return 1j
            if node.id.startswith("__p_") and node.id[4:] in env:
                return env[node.id[4:]]
            raise ValueError(f"unknown name {node.id} in {text!r}")
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp):
            a, b = ev(node.left), ev(node.right)
            ops = {ast.Add: lambda: a + b, ast.Sub: lambda: a - b, ast.Mult: lambda: a * b,
                   ast.Div: lambda: a / b, ast.Pow: lambda: a ** b}
            for k, f in ops.items():
                if isinstance(node.op, k):
                    return f()
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) \
                and node.func.id in _ALLOWED_FUNCS and len(node.args) == 1:
            return _ALLOWED_FUNCS[node.func.id](ev(node.args[0]))
        raise ValueError(f"unsupported expression {text!r}")

    return ev(tree)


def _split_params(s: str):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    if cur.strip():
        out.append(cur)
    return out


_APP = re.compile(r"^((?:(?:DAGGER|CONTROLLED)\s+)*)([A-Za-z_][A-Za-z0-9_\-]*)\s*(\((.*)\))?\s*(.*)$")


def parse(text: str) -> Program:
    prog = Program()
    defgates = {}  # name -> ("matrix", params, rows) | ("perm", perm)
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        raw = lines[i].split("#", 1)[0].rstrip()
        i += 1
        line = raw.strip()
        if not line:
            continue
        head = line.split()[0].upper()
        if head == "DECLARE":
            m = re.match(r"DECLARE\s+(\w+)\s+(\w+)(\[(\d+)\])?", line, re.I)
            if not m:
                raise ValueError(f"bad DECLARE: {line}")
            prog.memory[m.group(1)] = int(m.group(4) or 1)
            continue
        if head == "DEFGATE":
            m = re.match(r"DEFGATE\s+([\w\-]+)\s*(\(([^)]*)\))?\s*(AS\s+(\w+))?\s*:", line, re.I)
            if not m:
                raise ValueError(f"bad DEFGATE: {line}")
            name = m.group(1)
            params = [p.strip().lstrip("%") for p in (m.group(3) or "").split(",") if p.strip()]
            kind = (m.group(5) or "MATRIX").upper()
            body = []
            while i < len(lines) and (lines[i].startswith(" ") or lines[i].startswith("\t")):
                if lines[i].strip():
                    body.append(lines[i].strip())
                i += 1
            if kind == "PERMUTATION":
                perm = [int(x) for x in ",".join(body).split(",") if x.strip()]
                defgates[name] = ("perm", perm)
            elif kind == "MATRIX":
                defgates[name] = ("matrix", params, [_split_params(r) for r in body])
            else:
                raise ValueError(f"DEFGATE AS {kind} is not supported")
            continue
        if head == "MEASURE":
            parts = line.split()
            q = int(parts[1])
            mref = None
            if len(parts) > 2:
                mm = re.match(r"(\w+)(\[(\d+)\])?", parts[2])
                mref = (mm.group(1), int(mm.group(3) or 0))
            prog.instructions.append(Measure(q, mref))
            continue
        if head == "RESET":
            prog.instructions.append(Reset())
            continue
        if head in ("NOP", "HALT", "PRAGMA"):
            continue
        m = _APP.match(line)
        if not m:
            raise ValueError(f"cannot parse: {line}")
        mods = m.group(1).split()
        name = m.group(2)
        params = [eval_expr(p) for p in _split_params(m.group(4))] if m.group(3) else []
        args = [int(a) for a in m.group(5).split()]
        kind, perm = "dense", None
        if name in defgates:
            d = defgates[name]
            if d[0] == "perm":
                perm = d[1]
                kind = "perm"
                mat = np.zeros((len(perm), len(perm)), dtype=np.complex128)
                for j, p in enumerate(perm):
                    mat[j, p] = 1
            else:
                env = dict(zip(d[1], params))
                mat = np.array([[complex(eval_expr(e, env)) for e in row] for row in d[2]],
                               dtype=np.complex128)
        elif name in STANDARD_GATES:
            mat = gate_matrix(name, *params)
        else:
            raise KeyError(f"unknown gate {name}")
        for mod in reversed(mods):
            if mod.upper() == "DAGGER":
                mat = dagger(mat)
                kind, perm = "dense", None
            else:
                mat = controlled(mat)
                kind, perm = "dense", None
        if mat.shape[0] != 1 << len(args):
            raise ValueError(f"gate {name} applied to {len(args)} qubits")
        prog.instructions.append(GateApp(name, mat, args, kind, perm))
    return prog


def compile_measure_chains(instructions, n: int):
    """Replace contiguous MEASURE chains that cover all n qubits with a
    MeasureAll pseudo-instruction (src/compile-gate.lisp:552-599)."""
    out = []
    i = 0
    while i < len(instructions):
        j = i
        while j < len(instructions) and isinstance(instructions[j], Measure):
            j += 1
        chain = instructions[i:j]
        if chain and len(chain) >= n and {m.qubit for m in chain} >= set(range(n)):
            out.append(MeasureAll([(m.qubit, m.mref) for m in chain if m.mref is not None]))
            i = j
            continue
        if chain:
            out.extend(chain)
            i = j
        else:
            out.append(instructions[i])
            i += 1
    return out
