"""Layer drivers of the reference's workspace library (workspace/lib/haar.rs:103-210).

Unlike ``circuit::apply_bilayer`` (one measurement layer, one refactor sweep),
these measure the listed qubits one at a time, in list order, each with the
full refactor sweep of ``MPS::measure`` / ``measure_postsel``
(mps.rs:1471-1510).  Every call runs on the GPU through ``MPS``.

``unis`` is a ``UniLayer``: a list of ``(k, 4x4 matrix)``.  ``meas`` is a list
of ``Meas`` (``Meas.rand(k)``, or ``Meas.proj(k, outcome)`` for the
workspace's ``Postsel(k, bool)``).  ``us[j]`` is the uniform the j-th *random*
measurement of the list draws (the reference draws one per ``measure`` call).
Outcomes come back as ``Meas.proj`` values, as the reference returns
``Postsel``.
"""
from __future__ import annotations

from .gates import Meas


def _uniforms(us):
    it = iter(us if us is not None else ())

    def nxt():
        try:
            return float(next(it))
        except StopIteration:
            raise ValueError("one uniform per random measurement is needed") from None

    return nxt


def apply_main_layer(state, unis, meas, us=None):
    """``apply_main_layer`` (haar.rs:103-134)."""
    return apply_main_layer_probs(state, unis, meas, us)[0]


def apply_main_layer_probs(state, unis, meas, us=None):
    """``apply_main_layer_probs`` (haar.rs:136-166): (outcomes, [(k, prob)]),
    prob being the Born probability of the outcome before the projection."""
    for k, mat in unis:
        state.apply_unitary2(int(k), mat)
    nxt = _uniforms(us)
    outs, probs = [], []
    for m in meas:
        if m.is_rand():
            r = state.measure_prob(m.k, nxt())
            if r is None:  # out of range: the reference's unwrap panics here
                raise IndexError(f"qubit {m.k} out of range")
            o, p = r
        else:
            p = state.measure_postsel_prob(m.k, m.outcome)
            if p is None:
                raise IndexError(f"qubit {m.k} out of range")
            o = m.outcome
        outs.append(Meas.proj(m.k, o))
        probs.append((m.k, p))
    return outs, probs


def apply_probe_layer(state, unis, meas, target=None, us=None):
    """``apply_probe_layer`` (haar.rs:168-206): (outcomes, (p0, p1) at
    ``target`` or None).  As the reference's filter (haar.rs:188,
    ``target.is_none_or(|j| j == m.idx())``) is written, a target keeps only
    the measurements *at* the target (its comment says the opposite); the
    drop-in follows the code."""
    for k, mat in unis:
        state.apply_unitary2(int(k), mat)
    nxt = _uniforms(us)
    outs = []
    for m in meas:
        if target is not None and m.k != target:
            continue
        if m.is_rand():
            o = state.measure(m.k, nxt())
            if o is None:
                raise IndexError(f"qubit {m.k} out of range")
        else:
            state.measure_postsel(m.k, m.outcome)
            o = m.outcome
        outs.append(Meas.proj(m.k, o))
    probs = None
    if target is not None:
        p = state.probs(target)
        probs = None if p is None else (float(p[0]), float(p[1]))
    return outs, probs
