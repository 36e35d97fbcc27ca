"""OpenQASM 2.0 front-end feeding the engine's compiled circuits.

The reference reads OpenQASM through a generated parser (qgate/openqasm/,
built on ply, which translates a program into qgate.script calls).  This
module parses OpenQASM 2.0 itself -- a hand-written lexer and recursive-descent
parser -- and lowers a program straight to the engine's gate table: every
gate becomes a 2x2 complex matrix on a target lane with control lanes, the
form `qgate_gb300.compiled.CompiledCircuit` and the runtime's
apply_controlled_gate take.

Supported: `OPENQASM 2.0;`, `include "qelib1.inc";` (the standard gate names
become available; they are implemented here from their definitions as
matrices), `qreg` / `creg`, the built-ins `U(theta, phi, lambda)` and `CX`,
user `gate` definitions with parameters (expanded as macros), register
broadcasting, expressions (+ - * / ^, unary -, pi, sin cos tan exp ln sqrt),
`barrier` (ignored), `measure`, `reset` and `if (creg == n) qop` anywhere,
as the reference's grammar accepts them (qgate/openqasm/yacc.py:74, :82-91,
:115-124).  `opaque` raises QasmError.

A program whose measurements all come after the gates of their qubits (and
that has no `if` and no reset of a used qubit) is static: its gates form one
compiled circuit (`compile()`) and its measurements are drawn from the final
state by a sampling pool (`sample()`).  Any program runs shot by shot with
`run()`, which executes the gates in compiled segments and the measurements,
resets and conditions in between with the runtime's own operations, under
the reference's rules (qgate/simulator/rop_executor.py:36-53,
qgate/simulator/model_executor.py:117-136): a measurement draws u and
returns 0 iff u < Pr(qubit = 0), then collapses the state (decohere); a reset
needs the qubit measured and moves a |1> outcome back to |0> (apply_reset);
`if (c == n)` runs its operation when the register c, read as an integer with
c[0] the least significant bit, equals n.

Conventions (OpenQASM 2.0): U(t, p, l) = [[cos(t/2), -e^{il} sin(t/2)],
[e^{ip} sin(t/2), e^{i(p+l)} cos(t/2)]]; u1(l) = diag(1, e^{il});
rz(p) = u1(p); crz(l) is the controlled diag(e^{-il/2}, e^{il/2}); cu3 and
cu1 are the controlled u3 and u1 with no extra phase.  Lane i of the engine
state is qubit i in declaration order of the qregs.

The reference's translation maps `U`, `u3` and `u2` to qgate's U3 and U2
(qgate/openqasm/formatter.py:71-76), whose matrices carry an extra global
phase e^{-i(phi+lambda)/2} (qgate/simulator/src/GateMatrix.cpp:13-15): the
same program gives the same probabilities, samples and measurement outcomes
here, and amplitudes that differ from the reference's by that global phase.
Expressions follow OpenQASM (`^` is a power, right-associative and binding
tighter than unary minus: -2^2 = -4); the reference pastes them into generated Python source, where `^`
is an integer XOR.
"""
import math
import re

import numpy as np


class QasmError(ValueError):
    pass


# ------------------------------------------------------------------ lexer

_TOKEN = re.compile(r'''
    (?P<ws>[ \t\r\n]+|//[^\n]*)
  | (?P<real>(?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)
  | (?P<int>\d+)
  | (?P<str>"[^"\n]*")
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>->|==|[\[\](){};,+\-*/^])
''', re.X)


def _lex(text):
    toks, pos, line = [], 0, 1
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise QasmError('line %d: unexpected character %r' % (line, text[pos]))
        kind = m.lastgroup
        val = m.group()
        if kind != 'ws':
            toks.append((kind, val, line))
        line += val.count('\n')
        pos = m.end()
    toks.append(('eof', '', line))
    return toks


# ------------------------------------------------------------------ gate matrices

def _u(theta, phi, lam):
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return np.array([[c, -np.exp(1j * lam) * s],
                     [np.exp(1j * phi) * s, np.exp(1j * (phi + lam)) * c]], np.complex128)


def _u1(lam):
    return np.array([[1, 0], [0, np.exp(1j * lam)]], np.complex128)


# Upper bound on the gates one program may expand to: user gates that call
# each other several times grow exponentially with nesting depth, and this
# stops such a program with a parse error instead of exhausting host memory.
MAX_OPS = 50_000_000

_X = np.array([[0, 1], [1, 0]], np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], np.complex128)
_Z = np.array([[1, 0], [0, -1]], np.complex128)
_H = np.array([[1, 1], [1, -1]], np.complex128) / math.sqrt(2)
_I = np.eye(2, dtype=np.complex128)


def _rx(t):
    return _u(t, -math.pi / 2, math.pi / 2)


def _crz_diag(lam):
    return np.array([[np.exp(-0.5j * lam), 0], [0, np.exp(0.5j * lam)]], np.complex128)


# name -> (parameters, qubits, lowering(params) -> [(matrix, qubit index of the
# target, qubit indices of the controls)]) with qubit indices into the gate's
# argument list.
def _one(f):
    return lambda p: [(f(*p), 0, ())]


def _ctrl(f):
    return lambda p: [(f(*p), 1, (0,))]


_STD = {
    'u3': (3, 1, _one(_u)),
    'u2': (2, 1, _one(lambda p, l: _u(math.pi / 2, p, l))),
    'u1': (1, 1, _one(_u1)),
    'u': (3, 1, _one(_u)),
    'p': (1, 1, _one(_u1)),
    'u0': (1, 1, _one(lambda g: _I)),
    'id': (0, 1, _one(lambda: _I)),
    'x': (0, 1, _one(lambda: _X)),
    'y': (0, 1, _one(lambda: _Y)),
    'z': (0, 1, _one(lambda: _Z)),
    'h': (0, 1, _one(lambda: _H)),
    's': (0, 1, _one(lambda: _u1(math.pi / 2))),
    'sdg': (0, 1, _one(lambda: _u1(-math.pi / 2))),
    't': (0, 1, _one(lambda: _u1(math.pi / 4))),
    'tdg': (0, 1, _one(lambda: _u1(-math.pi / 4))),
    'rx': (1, 1, _one(_rx)),
    'ry': (1, 1, _one(lambda t: _u(t, 0., 0.))),
    'rz': (1, 1, _one(_u1)),
    'sx': (0, 1, _one(lambda: _rx(math.pi / 2))),
    'sxdg': (0, 1, _one(lambda: _rx(-math.pi / 2))),
    'cx': (0, 2, _ctrl(lambda: _X)),
    'cy': (0, 2, _ctrl(lambda: _Y)),
    'cz': (0, 2, _ctrl(lambda: _Z)),
    'ch': (0, 2, _ctrl(lambda: _H)),
    'crx': (1, 2, _ctrl(_rx)),
    'cry': (1, 2, _ctrl(lambda t: _u(t, 0., 0.))),
    'crz': (1, 2, _ctrl(_crz_diag)),
    'cu1': (1, 2, _ctrl(_u1)),
    'cp': (1, 2, _ctrl(_u1)),
    'cu3': (3, 2, _ctrl(_u)),
    'cu': (4, 2, _ctrl(lambda t, p, l, g: np.exp(1j * g) * _u(t, p, l))),
    'swap': (0, 2, lambda p: [(_X, 1, (0,)), (_X, 0, (1,)), (_X, 1, (0,))]),
    'rzz': (1, 2, lambda p: [(_X, 1, (0,)), (_u1(p[0]), 1, ()), (_X, 1, (0,))]),
    'ccx': (0, 3, lambda p: [(_X, 2, (0, 1))]),
    'cswap': (0, 3, lambda p: [(_X, 1, (2,)), (_X, 2, (0, 1)), (_X, 1, (2,))]),
}


# ------------------------------------------------------------------ expressions

_FUNCS = {'sin': math.sin, 'cos': math.cos, 'tan': math.tan, 'exp': math.exp,
          'ln': math.log, 'sqrt': math.sqrt}


class _Parser:
    def __init__(self, text):
        self.toks = _lex(text)
        self.i = 0
        self.qregs = {}      # name -> (first lane, size)
        self.cregs = {}      # name -> (first clbit, size)
        self.n_qubits = 0
        self.n_clbits = 0
        self.gates = {}      # user gates: name -> (params, qargs, body tokens)
        self.std = False
        self.ops = []        # (matrix, target, controls)
        self.items = []      # the program: ('g', matrix, target, controls),
        #                      ('m', qubit, clbit), ('r', qubit),
        #                      ('if', first clbit, size, value, [items])
        self.measured = {}   # qubit -> clbit
        self.meas_order = []  # (qubit, clbit) in program order
        self.touched = set()
        self.flags = {'dynamic': False}
        self.depth = 0       # nesting of user-gate expansion

    # -- token helpers
    def peek(self, k=0):
        return self.toks[self.i + k]

    def next(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def error(self, msg, tok=None):
        tok = tok or self.peek()
        raise QasmError('line %d: %s' % (tok[2], msg))

    def expect(self, val=None, kind=None):
        t = self.next()
        if (val is not None and t[1] != val) or (kind is not None and t[0] != kind):
            self.error('expected %s, found %r' % (val or kind, t[1]), t)
        return t

    def accept(self, val):
        if self.peek()[1] == val and self.peek()[0] in ('op', 'id'):
            self.i += 1
            return True
        return False

    # -- expressions over the gate parameters in `env`
    def expr(self, env):
        v = self.term(env)
        while self.peek()[1] in ('+', '-') and self.peek()[0] == 'op':
            op = self.next()[1]
            r = self.term(env)
            v = v + r if op == '+' else v - r
        return v

    def term(self, env):
        v = self.factor(env)
        while self.peek()[1] in ('*', '/') and self.peek()[0] == 'op':
            op = self.next()[1]
            r = self.factor(env)
            if op == '*':
                v *= r
            else:
                if r == 0:
                    self.error('division by zero')
                v /= r
        return v

    def factor(self, env):
        if self.peek()[1] == '-' and self.peek()[0] == 'op':
            self.next()
            return -self.factor(env)
        if self.peek()[1] == '+' and self.peek()[0] == 'op':
            self.next()
            return self.factor(env)
        base = self.atom(env)
        if self.peek()[1] == '^' and self.peek()[0] == 'op':
            self.next()
            return base ** self.factor(env)  # right-associative
        return base

    def atom(self, env):
        t = self.next()
        if t[0] in ('real', 'int'):
            return float(t[1])
        if t[0] == 'id':
            if t[1] == 'pi':
                return math.pi
            if t[1] in _FUNCS:
                self.expect('(')
                a = self.expr(env)
                self.expect(')')
                try:
                    return _FUNCS[t[1]](a)
                except ValueError:
                    self.error('%s(%g) is undefined' % (t[1], a), t)
            if t[1] in env:
                return env[t[1]]
            self.error('unknown parameter %r' % t[1], t)
        if t[1] == '(':
            v = self.expr(env)
            self.expect(')')
            return v
        self.error('unexpected %r in an expression' % t[1], t)

    def explist(self, env):
        vals = [self.expr(env)]
        while self.accept(','):
            vals.append(self.expr(env))
        return vals

    # -- program
    def program(self):
        self.expect('OPENQASM')
        v = self.next()
        if v[1] not in ('2.0', '2'):
            self.error('only OpenQASM 2.0 is supported', v)
        self.expect(';')
        while self.peek()[0] != 'eof':
            self.statement()
        return self

    def statement(self):
        t = self.peek()
        kw = t[1] if t[0] == 'id' else None
        if kw == 'include':
            self.next()
            f = self.expect(kind='str')[1][1:-1]
            if f != 'qelib1.inc':
                self.error('only "qelib1.inc" can be included', t)
            self.std = True
            self.expect(';')
        elif kw in ('qreg', 'creg'):
            self.next()
            name = self.expect(kind='id')[1]
            self.expect('[')
            size = int(self.expect(kind='int')[1])
            self.expect(']')
            self.expect(';')
            if name in self.qregs or name in self.cregs:
                self.error('register %r declared twice' % name, t)
            if size <= 0:
                self.error('register %r has no bits' % name, t)
            if kw == 'qreg':
                self.qregs[name] = (self.n_qubits, size)
                self.n_qubits += size
            else:
                self.cregs[name] = (self.n_clbits, size)
                self.n_clbits += size
        elif kw == 'gate':
            self.gate_decl()
        elif kw == 'opaque':
            self.error('opaque gates cannot be simulated', t)
        elif kw == 'if':
            self.next()
            self.expect('(')
            c = self.expect(kind='id')
            if c[1] not in self.cregs:
                self.error('unknown creg %r' % c[1], c)
            self.expect('==')
            value = int(self.expect(kind='int')[1])
            self.expect(')')
            first, size = self.cregs[c[1]]
            body = []
            outer, self.items = self.items, body
            try:
                self.qop()
            finally:
                self.items = outer
            self.flags['dynamic'] = True
            self.items.append(('if', first, size, value, body))
        elif kw == 'barrier':
            self.next()
            self.args_any()
            self.expect(';')
        else:
            self.qop()

    def qop(self):
        """One quantum operation: a gate application, `measure` or `reset`."""
        t = self.peek()
        kw = t[1] if t[0] == 'id' else None
        if kw == 'measure':
            self.next()
            qs = self.argument(self.qregs, 'qreg')
            self.expect('->')
            cs = self.argument(self.cregs, 'creg')
            self.expect(';')
            if len(qs) != len(cs):
                self.error('measure of registers of different sizes', t)
            for q, c in zip(qs, cs):
                self.measured[q] = c
                self.meas_order.append((q, c))
                self.items.append(('m', q, c))
        elif kw == 'reset':
            self.next()
            qs = self.argument(self.qregs, 'qreg')
            self.expect(';')
            for q in qs:
                if q in self.touched or q in self.measured:
                    self.flags['dynamic'] = True
                self.items.append(('r', q))
        elif kw in ('if', 'barrier', 'qreg', 'creg', 'gate', 'opaque', 'include'):
            self.error('%r cannot follow if (...)' % kw, t)
        else:
            self.gate_call({}, None)

    def argument(self, regs, what):
        t = self.expect(kind='id')
        if t[1] not in regs:
            self.error('unknown %s %r' % (what, t[1]), t)
        first, size = regs[t[1]]
        if self.accept('['):
            k = int(self.expect(kind='int')[1])
            self.expect(']')
            if k >= size:
                self.error('%s[%d] out of range (size %d)' % (t[1], k, size), t)
            return [first + k]
        return list(range(first, first + size))

    def args_any(self):
        out = [self.argument(self.qregs, 'qreg')]
        while self.accept(','):
            out.append(self.argument(self.qregs, 'qreg'))
        return out

    def gate_decl(self):
        t = self.next()
        name = self.expect(kind='id')[1]
        if name in self.gates or name in ('U', 'CX') or (self.std and name in _STD):
            self.error('gate %r defined twice' % name, t)
        params = []
        if self.accept('('):
            if not self.accept(')'):
                params.append(self.expect(kind='id')[1])
                while self.accept(','):
                    params.append(self.expect(kind='id')[1])
                self.expect(')')
        qargs = [self.expect(kind='id')[1]]
        while self.accept(','):
            qargs.append(self.expect(kind='id')[1])
        if len(set(qargs)) != len(qargs):
            self.error('gate %r repeats a qubit argument' % name, t)
        self.expect('{')
        start = self.i
        depth = 1
        while depth:
            tk = self.next()
            if tk[0] == 'eof':
                self.error('unterminated gate body', t)
            if tk[1] == '{':
                depth += 1
            elif tk[1] == '}':
                depth -= 1
        self.gates[name] = (params, qargs, self.toks[start:self.i - 1] + [('eof', '', tk[2])])

    # -- gate application: at top level (`scope` None, qubit args are
    # registers) or inside a gate body (`scope` maps qubit names to lanes)
    def gate_call(self, env, scope):
        t = self.next()
        if t[0] != 'id':
            self.error('expected a statement, found %r' % t[1], t)
        name = t[1]
        if name == 'barrier' and scope is not None:
            while self.peek()[1] != ';':
                self.next()
            self.expect(';')
            return
        params = []
        if self.accept('('):
            if not self.accept(')'):
                params = self.explist(env)
                self.expect(')')
        if scope is None:
            args = self.args_any()
        else:
            args = [[self.body_qubit(scope)]]
            while self.accept(','):
                args.append([self.body_qubit(scope)])
        self.expect(';')
        sizes = {len(a) for a in args if len(a) > 1}
        if len(sizes) > 1:
            self.error('registers of different sizes in one gate application', t)
        width = sizes.pop() if sizes else 1
        for k in range(width):
            lanes = [a[k] if len(a) > 1 else a[0] for a in args]
            if len(set(lanes)) != len(lanes):
                self.error('gate %r applied to one qubit twice' % name, t)
            self.apply(name, params, lanes, t)

    def body_qubit(self, scope):
        t = self.expect(kind='id')
        if t[1] not in scope:
            self.error('unknown qubit %r in a gate body' % t[1], t)
        return scope[t[1]]

    def apply(self, name, params, lanes, tok):
        def emit(mat, target, controls):
            for q in (target,) + tuple(controls):
                if q in self.measured:
                    self.flags['dynamic'] = True  # a gate after a measurement
                self.touched.add(q)
            if len(self.ops) >= MAX_OPS:
                self.error('program expands to more than %d gates' % MAX_OPS, tok)
            self.ops.append((mat, target, tuple(controls)))
            self.items.append(('g', mat, target, tuple(controls)))

        def arity(np_, nq):
            if len(params) != np_ or len(lanes) != nq:
                self.error('%s takes %d parameters and %d qubits (got %d and %d)'
                           % (name, np_, nq, len(params), len(lanes)), tok)

        if name == 'U':
            arity(3, 1)
            emit(_u(*params), lanes[0], ())
        elif name == 'CX':
            arity(0, 2)
            emit(_X, lanes[1], (lanes[0],))
        elif name in self.gates:
            pnames, qnames, body = self.gates[name]
            arity(len(pnames), len(qnames))
            if self.depth >= 64:
                self.error('gate %r expands recursively' % name, tok)
            sub = _Parser.__new__(_Parser)
            sub.__dict__.update(self.__dict__)
            sub.toks, sub.i, sub.depth = body, 0, self.depth + 1
            env = dict(zip(pnames, params))
            scope = dict(zip(qnames, lanes))
            while sub.peek()[0] != 'eof':
                sub.gate_call(env, scope)
        elif self.std and name in _STD:
            np_, nq, lower = _STD[name]
            arity(np_, nq)
            for mat, t, cs in lower(params):
                emit(mat, lanes[t], tuple(lanes[c] for c in cs))
        else:
            self.error('unknown gate %r%s' % (name, '' if self.std else
                                              ' (standard gates need include "qelib1.inc")'), tok)


class QasmProgram:
    """A parsed OpenQASM 2.0 program: `n_qubits` lanes, `ops` as (2x2
    complex128 matrix, target lane, control lanes) in program order,
    `measurements` as (qubit, clbit) pairs by classical bit (a classical bit
    written twice keeps the later measurement), the register maps `qregs` /
    `cregs` (name -> (first index, size)), `items` (the whole program in
    order: ('g', matrix, target, controls), ('m', qubit, clbit),
    ('r', qubit), ('if', first clbit, size, value, [items])) and `dynamic`
    (True when measurements, resets or conditions sit between gates, so the
    program must run shot by shot with `run()`)."""

    def __init__(self, p):
        self.n_qubits = p.n_qubits
        self.n_clbits = p.n_clbits
        self.ops = p.ops
        self.items = p.items
        self.dynamic = p.flags['dynamic']
        last = {}
        for q, c in p.meas_order:
            last[c] = q
        self.measurements = sorted(((q, c) for c, q in last.items()), key=lambda qc: qc[1])
        self.qregs = dict(p.qregs)
        self.cregs = dict(p.cregs)
        self._segments = {}

    def _static_only(self, what):
        if self.dynamic:
            raise QasmError('%s needs a program without mid-circuit measurements, resets of '
                            'used qubits or if; run it shot by shot with run().' % what)

    def _plan(self, items, dtype, graph):
        """items with each run of consecutive gates replaced by one
        ('c', CompiledCircuit) segment (built once per precision)."""
        from .compiled import CompiledCircuit
        out, run = [], []

        def close():
            if run:
                out.append(('c', CompiledCircuit(dtype, [(m, False, t, list(c))
                                                         for m, t, c in run], graph=graph),
                            list(run)))
                run.clear()
        for it in items:
            if it[0] == 'g':
                run.append(it[1:])
                continue
            close()
            if it[0] == 'if':
                out.append(('if',) + it[1:4] + (self._plan(it[4], dtype, graph),))
            else:
                out.append(it)
        close()
        return out

    def run(self, qstates, randnum=None, graph=False, gate_runner=None):
        """Runs the program once on `qstates` (at least n_qubits lanes, in
        the state the program starts from -- normally |0...0>) and returns
        the classical register as an int (bit j = classical bit j).

        Gates run as compiled segments (CUDA-graph replay with graph=True);
        `gate_runner(qstates, [(matrix, target, controls)])`, when given,
        applies each segment instead.  A measurement takes the next uniform
        from `randnum` (an iterable of floats in [0, 1); numpy's global RNG
        when None, as the reference front-end draws them) and follows the
        reference: outcome 0 iff u < Pr(qubit = 0), then decohere; the
        qubit's lane state records the outcome.  A reset of a qubit measured
        1 applies the runtime's reset, of a qubit measured 0 or still in
        |0> (never touched, or reset since) does nothing; a reset of any
        other qubit raises RuntimeError('Qubit is not measured.'), as the
        reference does.  A gate on a measured qubit clears its lane state."""
        proc = qstates.processor
        if qstates.get_n_lanes() < self.n_qubits:
            raise QasmError('the program has %d qubits, the state %d lanes.'
                            % (self.n_qubits, qstates.get_n_lanes()))
        if gate_runner is None:
            key = (proc.dtype, bool(graph))
            if key not in self._segments:
                self._segments[key] = self._plan(self.items, proc.dtype, graph)
            prog = self._segments[key]
        else:
            prog = self._plan_host(self.items)
        uniforms = iter(randnum) if randnum is not None else None
        clbits = [0] * self.n_clbits
        lane_state = {}
        known_zero = set(range(self.n_qubits))

        def execute(items):
            for it in items:
                kind = it[0]
                if kind in ('c', 'h'):
                    for _, t, c in it[2]:
                        for q in (t,) + tuple(c):
                            lane_state.pop(q, None)
                            known_zero.discard(q)
                    if kind == 'c':
                        it[1].run(qstates)
                    else:
                        gate_runner(qstates, it[2])
                elif kind == 'm':
                    q, c = it[1], it[2]
                    p0 = proc.calc_probability(qstates, q)
                    u = next(uniforms) if uniforms is not None else np.random.random_sample()
                    v = 0 if u < p0 else 1
                    proc.decohere(v, p0, qstates, q)
                    lane_state[q] = v
                    clbits[c] = v
                    if v == 0:
                        known_zero.add(q)
                    else:
                        known_zero.discard(q)
                elif kind == 'r':
                    q = it[1]
                    v = lane_state.get(q, -1)
                    if v == 1:
                        proc.apply_reset(qstates, q)
                        del lane_state[q]
                    elif v == -1 and q not in known_zero:
                        raise RuntimeError('Qubit is not measured.')
                    known_zero.add(q)
                elif kind == 'if':
                    first, size, value, body = it[1:]
                    reg = sum(clbits[first + k] << k for k in range(size))
                    if reg == value:
                        execute(body)

        execute(prog)
        for q in range(self.n_qubits):
            if hasattr(qstates, 'set_lane_state'):
                qstates.set_lane_state(q, lane_state.get(q, -1))
        return sum(b << k for k, b in enumerate(clbits))

    def _plan_host(self, items):
        out, run = [], []
        for it in items:
            if it[0] == 'g':
                run.append(it[1:])
                continue
            if run:
                out.append(('h', None, list(run)))
                run = []
            if it[0] == 'if':
                out.append(('if',) + it[1:4] + (self._plan_host(it[4]),))
            else:
                out.append(it)
        if run:
            out.append(('h', None, list(run)))
        return out

    def shots(self, rt, n_shots, dtype=np.float32, randnum=None, graph=True):
        """Runs the program `n_shots` times from |0...0> on one states object
        of the runtime `rt` (reset between shots) and returns the classical
        registers (int64, bit j = classical bit j).  `randnum` supplies the
        measurements' uniforms in order across all shots."""
        qs = rt.create_qubit_states(dtype)
        qs.processor.initialize_qubit_states(qs, self.n_qubits)
        uniforms = iter(randnum) if randnum is not None else None
        out = np.zeros(n_shots, np.int64)
        try:
            for k in range(n_shots):
                qs.processor.reset_qubit_states(qs)
                out[k] = self.run(qs, uniforms, graph=graph)
        finally:
            qs.delete()
        return out

    def delete(self):
        """Frees the compiled segments built by run()."""
        def free(items):
            for it in items:
                if it[0] == 'c':
                    it[1].delete()
                elif it[0] == 'if':
                    free(it[4])
        for prog in self._segments.values():
            free(prog)
        self._segments.clear()

    def gates(self):
        """The ops in the form CompiledCircuit and apply_controlled_gate take:
        (matrix, adjoint flag, target lane, control lanes)."""
        return [(m, False, t, list(c)) for m, t, c in self.ops]

    def sample(self, rt, qstates, shots, randnum=None):
        """Draws `shots` outcomes of the program's measurements from
        `qstates` (its state after the program ran), through the runtime's
        sampling pool over the measured lanes (the other lanes summed out).
        Returns int64 values with bit j = classical bit j; `randnum` are the
        pool's uniforms (numpy's when None).  Static programs only."""
        self._static_only('sample()')
        if not self.measurements:
            raise QasmError('the program measures nothing.')
        from .circuit import Lane
        n = qstates.get_n_lanes()
        qubits = sorted({q for q, _ in self.measurements})
        if qubits[-1] >= n:
            raise QasmError('the program measures qubit %d of a %d-lane state.' % (qubits[-1], n))
        pos = {q: k for k, q in enumerate(qubits)}
        lanes = [Lane(l, pos.get(l, -1)) for l in range(n)]
        getter = rt.create_qubits_states_getter(qstates.processor.dtype)
        pool = getter.create_sampling_pool(list(range(len(qubits))), len(qubits),
                                           n - len(qubits), [(qstates, lanes)], [])
        try:
            idx = np.asarray(pool.sample(shots, randnum).intarray, np.int64)
        finally:
            pool.delete()
        out = np.zeros(len(idx), np.int64)
        for q, c in self.measurements:
            out |= ((idx >> pos[q]) & 1) << c
        return out

    def compile(self, dtype=np.float32, graph=True):
        """A CompiledCircuit of the program's gates (complex64 for float32).
        Static programs only."""
        self._static_only('compile()')
        from .compiled import CompiledCircuit
        return CompiledCircuit(dtype, self.gates(), graph=graph)


def parse(text):
    """Parses OpenQASM 2.0 source into a QasmProgram (QasmError on syntax
    errors and on what the engine cannot run, such as opaque gates)."""
    return QasmProgram(_Parser(text).program())


def load(path):
    with open(path) as f:
        return parse(f.read())
