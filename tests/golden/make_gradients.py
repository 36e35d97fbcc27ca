"""Generates tests/golden/gradients_hea12.npz: parameter-shift gradients of a
hardware-efficient ansatz computed by the reference itself.

Run where the reference sources and its CPU runtime are built
(`make -C oracle ref`):

    python tests/golden/make_gradients.py [--ref /path/to/reference]

Circuit: 12 qubits, 12 layers of Ry(theta) and Rz(theta) on every qubit
followed by a CX ring ctrl(q_i).X(q_{i+1 mod 12}) -- the structure of the
24-qubit adjoint benchmark at a size the reference's CPU runtime runs 577
times in seconds; 288 parameters uniform(-pi, pi) from default_rng(31).
Observable H = -sum_{i<11} Z_i Z_{i+1} - 0.7 sum_i X_i (open chain).  Each
energy is one `sim.run` on the reference's C++ CPU runtime in complex128,
<P> = 2 Pr(P = +1) - 1 from its own Pauli probabilities (`prob(ref, paulis)`,
qgate/model/pauli_gates_diagonalizer.py).  Ry/Rz(theta) = exp(-i theta/2 P)
(qgate/simulator/src/GateMatrix.cpp), so dE/dtheta = (E(theta + pi/2) -
E(theta - pi/2)) / 2.  Written: params (288,), energy (), grad (288,).
"""
import argparse
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_import import reference_root  # noqa: E402

N, LAYERS = 12, 12


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=reference_root())
    args = ap.parse_args()
    from oracle.ref_import import import_reference
    qgate = import_reference(args.ref)
    from qgate.script import new_qregs, new_references, prob, ctrl, X, Z, Ry, Rz

    params = np.random.default_rng(31).uniform(-math.pi, math.pi, 2 * N * LAYERS)
    q = new_qregs(N)
    terms = [(-1.0, [Z(q[i]), Z(q[i + 1])]) for i in range(N - 1)]
    terms += [(-0.7, [X(q[i])]) for i in range(N)]

    def energy(theta):
        c = []
        p = 0
        for _ in range(LAYERS):
            for i in range(N):
                c.append(Ry(float(theta[p]))(q[i]))
                p += 1
            for i in range(N):
                c.append(Rz(float(theta[p]))(q[i]))
                p += 1
            for i in range(N):
                c.append(ctrl(q[i]).X(q[(i + 1) % N]))
        refs = new_references(len(terms))
        c += [prob(r, paulis) for r, (_, paulis) in zip(refs, terms)]
        sim = qgate.simulator.cpu(circuit_prep=qgate.prefs.one_static, dtype=np.float64)
        sim.run(c)
        e = sum(coef * (2. * sim.values.get(r) - 1.) for r, (coef, _) in zip(refs, terms))
        sim.terminate()
        return e

    t0 = time.time()
    e0 = energy(params)
    grad = np.empty(len(params))
    for k in range(len(params)):
        plus, minus = params.copy(), params.copy()
        plus[k] += math.pi / 2
        minus[k] -= math.pi / 2
        grad[k] = 0.5 * (energy(plus) - energy(minus))
    np.savez_compressed(os.path.join(HERE, 'gradients_hea12.npz'), params=params,
                        energy=np.float64(e0), grad=grad)
    print('E = %.12f, |grad| = %.6f, %d runs in %.1f s' % (e0, np.linalg.norm(grad),
                                                          2 * len(params) + 1, time.time() - t0))


if __name__ == '__main__':
    main()
