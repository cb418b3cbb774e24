"""Straight-line programs: systems given as a sequence of operations instead of term tables.

The reference evaluates every system through ModelKit's ``InstructionSequence``
(src/model_kit/instruction_sequence.jl:1-27): a tape of constants, variables and instruction
outputs, each instruction an op of ``OpType`` (src/model_kit/operations.jl:5-49) on up to four
tape slots. ``Program`` is that tape; ``variables(n)`` returns tracing variables whose
arithmetic records instructions (a node used twice is computed once), so a structured system
— products of linear forms, determinants, rational expressions — is passed without expanding
it. ``hc_set_slp`` turns the program into CUDA C and compiles it with NVRTC together with the
tracking kernel (the cubin is cached by hash, as the reference caches compiled systems,
src/model_kit/compiled_system_homotopy.jl:39-57).

    x = variables(3)
    F = Program([x[0] * x[1] - 1, (x[0] + x[1]) ** 2 - x[2], x[2] / (x[0] - 3) + 2], degrees=[2, 2, 2])
    H = slp_homotopy(F, gamma)              # γ t G + (1 - t) F, G the total-degree start system
    T = EndgameTracker(H); T.track_arrays(total_degree_start_solutions(H.degrees))

A program may also have parameters (``variables_and_parameters``), entering it in any way the
ops allow; ``slp_parameter_homotopy(F, p, q)`` is then the reference's ParameterHomotopy
H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44), tracked from
solutions of F(x; p) at t = 1 to t = 0 (``hc_set_slp_parameter_homotopy``); ``F.fixed(p)`` is
F(·; p) as a parameter-free program (``fix_parameters``), e.g. to find start solutions by a
total-degree solve.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

# OpType values (src/model_kit/operations.jl:5-49), as in include/hcgpu.h
OPS = ["STOP", "CB", "ACOS", "ASIN", "COS", "COSH", "EXP", "INV", "INV_NOT_ZERO", "INVSQR", "NEG", "SIN", "SINH",
       "SQR", "SQRT", "TAN", "TANH", "IDENTITY", "ADD", "DIV", "MUL", "SUB", "POW_INT", "POW", "ADD3", "MUL3",
       "MULADD", "MULSUB", "SUBMUL", "ADD4", "MUL4", "MULMULADD", "MULMULSUB"]
OP = {name: k for k, name in enumerate(OPS)}
ARITY = {**{o: 1 for o in ("CB", "ACOS", "ASIN", "COS", "COSH", "EXP", "INV", "INV_NOT_ZERO", "INVSQR", "NEG",
                            "SIN", "SINH", "SQR", "SQRT", "TAN", "TANH", "IDENTITY")},
         **{o: 2 for o in ("ADD", "DIV", "MUL", "SUB", "POW_INT", "POW")},
         **{o: 3 for o in ("ADD3", "MUL3", "MULADD", "MULSUB", "SUBMUL")},
         **{o: 4 for o in ("ADD4", "MUL4", "MULMULADD", "MULMULSUB")}}

INSTR_DTYPE = np.dtype([("input", np.int32, 4), ("op", np.int32), ("output", np.int32)])


class _Tape:
    """Records instructions; nodes are ('c', k) constants, ('x', j) variables, ('p', k)
    parameters, ('t', k) outputs."""

    def __init__(self, n, nparams=0):
        self.n = n
        self.np = nparams
        self.consts: list = []
        self.cindex: dict = {}
        self.instr: list = []  # (op name, input nodes, exponent or None)
        self.memo: dict = {}

    def const(self, c) -> tuple:
        c = complex(c)
        key = (c.real, c.imag)
        if key not in self.cindex:
            self.cindex[key] = len(self.consts)
            self.consts.append(c)
        return ("c", self.cindex[key])

    def op(self, name, inputs, p=None) -> tuple:
        key = (name, tuple(inputs), p)
        if key not in self.memo:
            self.instr.append((name, tuple(inputs), p))
            self.memo[key] = ("t", len(self.instr) - 1)
        return self.memo[key]


class Expr:
    """A traced value: arithmetic with other Exprs or numbers records instructions."""

    __array_priority__ = 1000

    def __init__(self, tape: _Tape, node: tuple):
        self.tape, self.node = tape, node

    def _wrap(self, v) -> "Expr":
        if isinstance(v, Expr):
            if v.tape is not self.tape:
                raise ValueError("expressions of different programs")
            return v
        return Expr(self.tape, self.tape.const(v))

    def _op(self, name, *args, p=None) -> "Expr":
        return Expr(self.tape, self.tape.op(name, [a.node for a in args], p))

    def __add__(self, o):
        return self._op("ADD", self, self._wrap(o))

    def __radd__(self, o):
        return self._op("ADD", self._wrap(o), self)

    def __sub__(self, o):
        return self._op("SUB", self, self._wrap(o))

    def __rsub__(self, o):
        return self._op("SUB", self._wrap(o), self)

    def __mul__(self, o):
        return self._op("MUL", self, self._wrap(o))

    def __rmul__(self, o):
        return self._op("MUL", self._wrap(o), self)

    def __truediv__(self, o):
        return self._op("DIV", self, self._wrap(o))

    def __rtruediv__(self, o):
        return self._op("DIV", self._wrap(o), self)

    def __neg__(self):
        return self._op("NEG", self)

    def __pow__(self, p):
        p = int(p)
        if p == 2:
            return self._op("SQR", self)
        if p == 3:
            return self._op("CB", self)
        return self._op("POW_INT", self, p=p)


def variables(n: int):
    """n tracing variables x_1..x_n of a new program."""
    tape = _Tape(n)
    return [Expr(tape, ("x", j)) for j in range(n)]


def variables_and_parameters(n: int, m: int):
    """n tracing variables and m parameters of a new program (ModelKit's
    ``System(f, variables, parameters)``): returns (x, p)."""
    tape = _Tape(n, m)
    return [Expr(tape, ("x", j)) for j in range(n)], [Expr(tape, ("p", k)) for k in range(m)]


def op(name: str, *args: Expr, p: Optional[int] = None) -> Expr:
    """Record any ModelKit op by name, e.g. op("MULADD", a, b, c) = a*b + c, op("SQRT", a),
    op("POW_INT", a, p=-2)."""
    if name not in ARITY:
        raise ValueError(f"unknown op {name}")
    want = 1 if name == "POW_INT" else ARITY[name]
    if len(args) != want or (name == "POW_INT") != (p is not None):
        raise ValueError(f"{name} takes {want} inputs" + (" and an integer exponent p" if name == "POW_INT" else ""))
    return args[0]._op(name, *(args[0]._wrap(a) for a in args), p=p)


@dataclass
class Program:
    """A square system F: C^n → C^n as a straight-line program, with the degrees of its
    equations (the total-degree start system G_i = s_i (x_i^{D_i} - 1) uses them; without
    parameters they default to the degrees ``degree_bounds`` finds)."""

    outputs: Sequence
    degrees: Optional[Sequence[int]] = None
    scaling: Optional[Sequence[float]] = None

    def __post_init__(self):
        outs = list(self.outputs)
        tape = next((o.tape for o in outs if isinstance(o, Expr)), None)
        if tape is None:
            raise ValueError("at least one output must depend on the variables")
        self.n = tape.n
        self.nparams = tape.np
        self._tape = tape
        self.outputs = [o if isinstance(o, Expr) else Expr(tape, tape.const(o)) for o in outs]
        if self.degrees is None:
            if self.nparams == 0:
                self.degrees = self.degree_bounds()
            else:  # no start system: the bounds where they exist (not used by the tracker)
                try:
                    self.degrees = self.degree_bounds()
                except ValueError:
                    self.degrees = [1] * self.n
        if len(outs) != self.n or len(self.degrees) != self.n:
            raise ValueError("a square system: n outputs and n degrees")
        if self.scaling is None:
            self.scaling = [1.0] * self.n

    @property
    def poff(self) -> int:
        """Tape slot of the first parameter (after the constants and the variables)."""
        return len(self._tape.consts) + self.n

    def arrays(self):
        """(instructions, constants re/im, variables_offset, tape_size, outputs) with constants at
        slots [0, nconst), variables next, then the parameters (``poff``), instruction outputs
        after them."""
        t = self._tape
        nc = len(t.consts)
        voff = nc
        poff = voff + self.n
        base = poff + self.nparams

        def slot(node):
            kind, k = node
            return {"c": k, "x": voff + k, "p": poff + k}.get(kind, base + k)

        ins = np.zeros(len(t.instr), dtype=INSTR_DTYPE)
        for k, (name, inputs, p) in enumerate(t.instr):
            row = [slot(v) for v in inputs] + [0] * (4 - len(inputs))
            if name == "POW_INT":
                row[1] = p
            ins[k]["input"] = row
            ins[k]["op"] = OP[name]
            ins[k]["output"] = base + k
        consts = np.array([[c.real, c.imag] for c in t.consts], dtype=np.float64).reshape(-1)
        outs = np.array([slot(o.node) for o in self.outputs], dtype=np.int32)
        return ins, consts, voff, base + len(t.instr), outs

    def evaluate(self, x, p=None):
        """F(x) (F(x; p) with parameters) with numpy complex arithmetic (the ops' semantics; for
        tests)."""
        t = self._tape
        vals = {}
        if self.nparams and p is None:
            raise ValueError(f"the program has {self.nparams} parameters")

        def v(node):
            kind, k = node
            if kind == "c":
                return t.consts[k]
            if kind == "x":
                return complex(x[k])
            if kind == "p":
                return complex(p[k])
            return vals[k]

        for k, (name, inputs, pw) in enumerate(t.instr):
            a = [v(i) for i in inputs]
            vals[k] = _apply(name, a, pw)
        return np.array([v(o.node) for o in self.outputs])


    def degree_bounds(self):
        """Upper bounds of the equations' degrees in x, by propagation through the ops (exact
        for the sums, products and powers of polynomials); raises ValueError where an output
        depends on the variables through a division, inverse or square root."""
        t = self._tape
        deg = {}

        def d(node):
            kind, k = node
            return 1 if kind == "x" else (0 if kind in ("c", "p") else deg[k])

        inf = float("inf")
        for k, (name, inputs, p) in enumerate(t.instr):
            a = [d(i) for i in inputs]
            if name in ("ADD", "SUB", "ADD3", "ADD4", "NEG", "IDENTITY"):
                deg[k] = max(a)
            elif name in ("MUL", "MUL3", "MUL4"):
                deg[k] = sum(a)
            elif name == "SQR":
                deg[k] = 2 * a[0]
            elif name == "CB":
                deg[k] = 3 * a[0]
            elif name == "POW_INT":
                deg[k] = p * a[0] if p >= 0 else (0 if a[0] == 0 else inf)
            elif name in ("MULADD", "MULSUB", "SUBMUL"):
                deg[k] = max(a[0] + a[1], a[2])
            elif name in ("MULMULADD", "MULMULSUB"):
                deg[k] = max(a[0] + a[1], a[2] + a[3])
            else:  # DIV, INV, INVSQR, INV_NOT_ZERO, SQRT: polynomial only in constants/parameters
                deg[k] = 0 if max(a) == 0 else inf
        out = [d(o.node) for o in self.outputs]
        if any(v == inf for v in out):
            raise ValueError("an equation is not polynomial in the variables: pass its degrees")
        return [max(int(v), 1) for v in out]

    def fixed(self, p, degrees=None) -> "Program":
        """F(·; p): the program with its parameters replaced by the constants p (fix_parameters,
        src/systems/fixed_parameter_system.jl)."""
        if not self.nparams:
            raise ValueError("the program has no parameters")
        p = [complex(v) for v in np.asarray(p, dtype=np.complex128).reshape(-1)]
        if len(p) != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {len(p)}")
        t = self._tape
        x = variables(self.n)
        tape = x[0].tape
        vals = {}

        def node(nd):
            kind, k = nd
            if kind == "c":
                return tape.const(t.consts[k])
            if kind == "x":
                return ("x", k)
            if kind == "p":
                return tape.const(p[k])
            return vals[k]

        for k, (name, inputs, pw) in enumerate(t.instr):
            vals[k] = tape.op(name, [node(i) for i in inputs], pw)
        outs = [Expr(tape, node(o.node)) for o in self.outputs]
        return Program(outs, degrees if degrees is not None else None, scaling=list(self.scaling))


def _apply(name, a, p):
    if name == "ADD":
        return a[0] + a[1]
    if name == "SUB":
        return a[0] - a[1]
    if name == "MUL":
        return a[0] * a[1]
    if name == "DIV":
        return a[0] / a[1]
    if name == "NEG":
        return -a[0]
    if name == "SQR":
        return a[0] * a[0]
    if name == "CB":
        return a[0] * a[0] * a[0]
    if name == "INV":
        return 1 / a[0]
    if name == "INV_NOT_ZERO":
        return a[0] if a[0] == 0 else 1 / a[0]
    if name == "INVSQR":
        return 1 / (a[0] * a[0])
    if name == "SQRT":
        return np.sqrt(complex(a[0]))
    if name == "IDENTITY":
        return a[0]
    if name == "POW_INT":
        return a[0] ** p
    if name == "ADD3":
        return a[0] + a[1] + a[2]
    if name == "MUL3":
        return a[0] * a[1] * a[2]
    if name == "MULADD":
        return a[0] * a[1] + a[2]
    if name == "MULSUB":
        return a[0] * a[1] - a[2]
    if name == "SUBMUL":
        return a[2] - a[0] * a[1]
    if name == "ADD4":
        return a[0] + a[1] + a[2] + a[3]
    if name == "MUL4":
        return a[0] * a[1] * a[2] * a[3]
    if name == "MULMULADD":
        return a[0] * a[1] + a[2] * a[3]
    if name == "MULMULSUB":
        return a[0] * a[1] - a[2] * a[3]
    raise ValueError(f"op {name} is not supported")


def from_system(F) -> Program:
    """A term-table System (systems.System) as a program: per equation, the sum of coefficient ×
    monomial with monomials built by POW_INT and MUL, shared between equations."""
    x = variables(F.n)
    degs = []
    outs = []
    mono_cache = {}

    def mono(e):
        e = tuple(int(v) for v in e)
        if e not in mono_cache:
            acc = None
            for j, p in enumerate(e):
                if p == 0:
                    continue
                f = x[j] if p == 1 else x[j] ** p
                acc = f if acc is None else acc * f
            mono_cache[e] = acc
        return mono_cache[e]

    for E, C in zip(F.exponents, F.coefficients):
        acc = None
        for e, c in zip(E, C):
            m = mono(e)
            term = complex(c) if m is None else (m if c == 1 else complex(c) * m)
            acc = term if acc is None else acc + term
        outs.append(acc if acc is not None else 0.0)
        degs.append(int(max(int(np.sum(e)) for e in E)) if len(E) else 1)
    # the start system's scaling of the reference (src/total_degree.jl:62)
    return Program(outs, degs, scaling=[float(np.max(np.abs(C))) for C in F.coefficients])


@dataclass
class SLPHomotopy:
    """γ t G(x) + (1 - t) F(x) with F a Program and G_i = s_i (x_i^{D_i} - 1)."""

    program: Program
    gamma: complex

    @property
    def n(self):
        return self.program.n

    @property
    def degrees(self):
        return list(self.program.degrees)


def slp_homotopy(F: Program, gamma) -> SLPHomotopy:
    return SLPHomotopy(F, complex(gamma))


@dataclass
class SLPParameterHomotopy:
    """H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44) with F a
    Program with parameters: p = start_parameters (t = 1), q = target_parameters (t = 0)."""

    program: Program
    start_parameters: np.ndarray
    target_parameters: np.ndarray

    def __post_init__(self):
        m = self.program.nparams
        if m == 0:
            raise ValueError("the program has no parameters")
        self.start_parameters = np.asarray(self.start_parameters, dtype=np.complex128).reshape(-1)
        self.target_parameters = np.asarray(self.target_parameters, dtype=np.complex128).reshape(-1)
        if self.start_parameters.shape[0] != m or self.target_parameters.shape[0] != m:
            raise ValueError(f"expected {m} start and target parameters")

    @property
    def n(self):
        return self.program.n

    def parameters(self, p, q) -> "SLPParameterHomotopy":
        """The same program with new (p, q) (parameters!, :56-62); on a tracker that already
        has the program this changes two small device arrays and compiles nothing."""
        return SLPParameterHomotopy(self.program, p, q)

    def evaluate(self, x, t):
        t = complex(t)
        return self.program.evaluate(x, t * self.start_parameters + (1 - t) * self.target_parameters)


def slp_parameter_homotopy(F: Program, start_parameters, target_parameters) -> SLPParameterHomotopy:
    return SLPParameterHomotopy(F, start_parameters, target_parameters)


class hc_slp(ct.Structure):
    _fields_ = [("n", ct.c_int32), ("ninstructions", ct.c_int32), ("instructions", ct.c_void_p),
                ("nconstants", ct.c_int32), ("constants", ct.c_void_p), ("variables_offset", ct.c_int32),
                ("tape_size", ct.c_int32), ("outputs", ct.c_void_p)]


def c_program(P: Program):
    """(hc_slp struct, degrees, scaling, arrays kept alive) for the C ABI."""
    ins, consts, voff, tape, outs = P.arrays()
    ins = np.ascontiguousarray(ins)
    consts = np.ascontiguousarray(consts if consts.size else np.zeros(2))
    outs = np.ascontiguousarray(outs)
    s = hc_slp(P.n, len(ins), ins.ctypes.data, len(consts) // 2 if len(P._tape.consts) else 0, consts.ctypes.data,
               voff, tape, outs.ctypes.data)
    deg = np.ascontiguousarray(np.asarray(P.degrees, dtype=np.int32))
    sc = np.ascontiguousarray(np.asarray(P.scaling, dtype=np.float64))
    return s, deg, sc, (ins, consts, outs)


def source(P: Program) -> str:
    """The CUDA C that hc_set_slp (hc_set_slp_parameter_homotopy for a program with
    parameters) compiles for P (no GPU needed)."""
    from . import _lib

    L = _lib.load()
    s, deg, sc, keep = c_program(P)
    n = ct.c_int64()

    def call(out, cap):
        if P.nparams:
            return L.hc_slp_parameter_source(ct.byref(s), P.nparams, P.poff, out, cap, ct.byref(n))
        return L.hc_slp_source(ct.byref(s), _lib.ptr(deg), _lib.ptr(sc), out, cap, ct.byref(n))

    _lib.check(call(None, 0))
    buf = ct.create_string_buffer(n.value + 1)
    _lib.check(call(buf, n.value + 1))
    return buf.value.decode()


# ------------------------------------------------------------------------------------------
# Structured systems: each as a program (unexpanded) and as its expanded term table
# ------------------------------------------------------------------------------------------
def products_of_linear_forms(n: int, d: int, seed: int):
    """F_i = ∏_{k<d} (a_ik · x + b_ik) - c_i with complex Gaussian a, b, c: degree d, Bézout
    d^n; expanded, each equation has up to C(n+d, d) terms, the program n·d·(n+1) operations."""
    from .systems import Poly, System, complex_gaussian
    from .systems import variables as poly_variables

    rng = np.random.Generator(np.random.PCG64(seed))
    A = complex_gaussian(rng, n * d * n).reshape(n, d, n)
    B = complex_gaussian(rng, n * d).reshape(n, d)
    Cc = complex_gaussian(rng, n)
    x = variables(n)
    X = poly_variables(n)
    outs, polys = [], []
    for i in range(n):
        f, p = None, Poly.const(1.0, n)
        for k in range(d):
            lin = complex(B[i, k]) + sum(complex(A[i, k, j]) * x[j] for j in range(n))
            f = lin if f is None else f * lin
            pl = Poly.const(complex(B[i, k]), n)
            for j in range(n):
                pl = pl + complex(A[i, k, j]) * X[j]
            p = p * pl
        outs.append(f - complex(Cc[i]))
        polys.append(p - complex(Cc[i]))
    return Program(outs, [d] * n), System.from_polys(polys)


def determinantal(n: int, k: int, seed: int):
    """F_i = det(M_i(x)) - 1 with M_i a k×k matrix of affine forms in x (complex Gaussian),
    the determinant taken by Gaussian elimination without pivoting — divisions (DIV), as a
    program would compute it — and expanded by the Leibniz formula for the term table.
    Degree k, Bézout k^n."""
    import itertools

    from .systems import Poly, System, complex_gaussian
    from .systems import variables as poly_variables

    rng = np.random.Generator(np.random.PCG64(seed))
    x = variables(n)
    X = poly_variables(n)
    outs, polys = [], []
    for i in range(n):
        C0 = complex_gaussian(rng, k * k).reshape(k, k)
        Cx = complex_gaussian(rng, k * k * n).reshape(k, k, n)
        M = [[complex(C0[r, c]) + sum(complex(Cx[r, c, j]) * x[j] for j in range(n)) for c in range(k)] for r in range(k)]
        P = [[Poly.const(complex(C0[r, c]), n) for c in range(k)] for r in range(k)]
        for r in range(k):
            for c in range(k):
                for j in range(n):
                    P[r][c] = P[r][c] + complex(Cx[r, c, j]) * X[j]
        # elimination: det = ∏ pivots
        det = None
        for c in range(k):
            piv = M[c][c]
            det = piv if det is None else det * piv
            for r in range(c + 1, k):
                f = M[r][c] / piv
                for q in range(c + 1, k):
                    M[r][q] = M[r][q] - f * M[c][q]
        outs.append(det - 1.0)
        # Leibniz
        pd = Poly.const(0.0, n)
        for perm in itertools.permutations(range(k)):
            sgn = 1
            for a in range(k):
                for b in range(a + 1, k):
                    if perm[a] > perm[b]:
                        sgn = -sgn
            term = Poly.const(float(sgn), n)
            for r in range(k):
                term = term * P[r][perm[r]]
            pd = pd + term
        polys.append(pd - 1.0)
    return Program(outs, [k] * n), System.from_polys(polys)


def disguised_ops(seed: int = 0):
    """Three quadrics written with every op the GPU evaluator supports (DIV, INV, INVSQR,
    INV_NOT_ZERO, SQRT, negative POW_INT, CB, and the 3- and 4-ary ops) in forms that
    simplify to polynomials away from their removable singularities; with the expanded table."""
    from .systems import Poly, System
    from .systems import variables as poly_variables

    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.normal(size=12) + 1j * rng.normal(size=12)
    x, y, z = variables(3)
    X, Y, Z = poly_variables(3)
    c = [complex(v) for v in a]
    f1 = op("MULADD", x, y, op("MULSUB", z, c[0], c[1])) + op("SUBMUL", x, c[2], op("IDENTITY", x * x))
    p1 = X * Y + (Z * c[0] - c[1]) + (X * X - X * c[2])
    # (x² y)/x = x y ; 1/(1/z) = z ; x³ · x⁻² = x ; sqrt(w)² = w ; invsqr(inv(y)) = y²
    f2 = (x * x * y) / x + op("INV", op("INV", z)) * c[3] + op("POW_INT", x, p=3) * op("POW_INT", x, p=-2) \
        + op("SQR", op("SQRT", y * c[4] + c[5])) + op("INVSQR", op("INV", y)) - c[6]
    p2 = X * Y + Z * c[3] + X + (Y * c[4] + c[5]) + Y * Y - c[6]
    f3 = op("ADD4", x * z, op("MUL3", y, c[7], z), op("MULMULADD", x, c[8], y, c[9]), -op("INV_NOT_ZERO", op("INV_NOT_ZERO", y))) \
        + op("MULMULSUB", z, z, x, c[10]) + op("ADD3", op("MUL4", x, c[11], 1.0, 1.0), op("NEG", z), 1.0) \
        + op("CB", x) / x
    p3 = X * Z + Y * c[7] * Z + (X * c[8] + Y * c[9]) - Y + (Z * Z - X * c[10]) + (X * c[11] - Z + 1.0) + X * X
    return Program([f1, f2, f3], [2, 2, 2]), System.from_polys([p1, p2, p3])
