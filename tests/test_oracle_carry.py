"""The oracle's step-size carry-over option (dt_carry), on the CPU.

* Without it the oracle is unchanged, and a first call with every carried
  step size 0 starts at dt * seed exactly as without it.
* A carried step size starts the next call at fmin(carry, dt): a call whose
  carry is the previous call's end state needs fewer attempts, and the
  results stay within the tolerance of the default path.
"""
import numpy as np

from mkpp_gb300 import workloads
from oracle.oracle import Oracle


def test_first_call_with_zero_carry_is_the_default():
    w = workloads.make("small_strato", 128)
    o = Oracle("small_strato")
    a = o.integrate(w.conc.copy(), w.dt, param=w.param)
    carry = np.zeros(128)
    b = o.integrate(w.conc.copy(), w.dt, param=w.param, dt_carry=carry)
    assert np.array_equal(a["conc"], b["conc"])
    assert np.array_equal(a["accepted"], b["accepted"]) and np.array_equal(a["rejected"], b["rejected"])
    assert np.all(carry > 0) and np.all(carry <= w.dt)


def test_carry_cuts_later_attempts_within_tolerance():
    w = workloads.make("small_strato", 128)
    o = Oracle("small_strato")
    plain, carried = w.conc.copy(), w.conc.copy()
    carry = np.zeros(128)
    n_plain = n_carry = 0
    for h in range(4):
        a = o.integrate(plain, w.dt, param=w.param_at(h))
        b = o.integrate(carried, w.dt, param=w.param_at(h), dt_carry=carry)
        plain, carried = a["conc"], b["conc"]
        if h:
            n_plain += int((a["accepted"] + a["rejected"]).sum())
            n_carry += int((b["accepted"] + b["rejected"]).sum())
    assert n_carry < 0.6 * n_plain
    tol = np.array(o.raw["rtol"])[:, None] * np.abs(plain) + np.array(o.raw["atol"])[:, None]
    assert np.all(np.abs(carried - plain) <= 10 * tol)
