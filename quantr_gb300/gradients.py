"""Energy and gradient API over the engine (no counterpart in quantr).

`energy_and_gradient(ansatz_or_program, a, b)` runs the circuit from |0...0> on the device and
returns E = <psi|H|psi> with H = sum_i a_i Z_i Z_{i+1} + sum_i b_i X_i (periodic) and dE/dtheta
for every gate by the adjoint method (qgpu_adjoint_grad). `parameter_shift` and
`finite_difference` compute the same gradient by repeated plain simulations on the device; they
are the comparison baselines.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native as nat
from ._native import KIND
from .program import Program

ROTATIONS = {KIND["Rx"], KIND["Ry"], KIND["Rz"], KIND["Phase"]}


def energy(handle: nat.Handle, prog: Program, a, b) -> float:
    handle.set_zero()
    handle.apply(prog.ops, prog.mats, prog.none)
    return handle.expectation_zzx(a, b)


def energy_and_gradient(handle: nat.Handle, prog: Program, a, b):
    handle.set_zero()
    return handle.adjoint_grad(prog.ops, prog.mats, prog.none, a, b)


def _shifted(prog: Program, g: int, delta: float) -> Program:
    ops = prog.ops.copy()
    ops["param"][g] += delta
    return Program(prog.n, ops, prog.mats, prog.none)


def parameter_shift(handle: nat.Handle, prog: Program, a, b) -> np.ndarray:
    """dE/dtheta = [E(theta + pi/2) - E(theta - pi/2)] / 2 for Rx/Ry/Rz (generator eigenvalues
    +-1/2); Phase is a global phase and gets 0."""
    grads = np.zeros(len(prog.ops))
    for g, k in enumerate(prog.ops["kind"]):
        if int(k) in ROTATIONS and int(k) != KIND["Phase"]:
            ep = energy(handle, _shifted(prog, g, math.pi / 2), a, b)
            em = energy(handle, _shifted(prog, g, -math.pi / 2), a, b)
            grads[g] = 0.5 * (ep - em)
    return grads


def finite_difference(handle: nat.Handle, prog: Program, a, b, h: float = 1e-6) -> np.ndarray:
    grads = np.zeros(len(prog.ops))
    for g, k in enumerate(prog.ops["kind"]):
        if int(k) in ROTATIONS:
            ep = energy(handle, _shifted(prog, g, h), a, b)
            em = energy(handle, _shifted(prog, g, -h), a, b)
            grads[g] = (ep - em) / (2.0 * h)
    return grads
