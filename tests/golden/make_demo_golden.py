"""Step-record fixtures (demo_*.npz) on the reference's own demo problems.

The reference ships no expected outputs for this path, but its demo program
src/cauchy_estimator.cpp holds fixed problems with fixed measurement
sequences (test_cauchy_2_state_moshe, _3_state_, _4_state_, _5_state_,
_3_state_moshe_3msmts, _four_state_two_pnoise, _4_state_2_msmts_moshe,
test_no_proc_noise: no process noise, 30 steps).
This script reads each demo's arrays (Phi, Gamma, H, beta, gamma, A0, p0, b0,
zs) and sizes (n, cmcc, pncc, p, steps) out of that file's text, runs the
reference estimator on them through oracle/ref_harness.cpp (serial build,
print_basic_info as the demos construct it, srand(seed) before the
constructor) and records every update as make_golden.py does.  Nothing of the
demo file is kept but the problem arrays and the reference's results.

Needs the reference sources:  python tests/golden/make_demo_golden.py
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import oracle  # noqa: E402
import make_golden  # noqa: E402

DEMOS = [
    ("demo_two_state_moshe", "test_cauchy_2_state_moshe", 301),
    ("demo_three_state_moshe", "test_cauchy_3_state_moshe", 302),
    ("demo_four_state_moshe", "test_cauchy_4_state_moshe", 303),
    ("demo_three_state_three_msmts", "test_cauchy_3_state_moshe_3msmts", 304),
    ("demo_four_state_two_pnoise", "test_cauchy_four_state_two_pnoise", 305),
    ("demo_four_state_two_msmts", "test_cauchy_4_state_2_msmts_moshe", 306),
    ("demo_five_state_moshe", "test_cauchy_5_state_moshe", 307),
    # srand(10) before the constructor, as the demo seeds it
    ("demo_no_process_noise", "test_no_proc_noise", 10),
]


def _strip_comments(text):
    """C comments removed in reading order (a '/*' inside a '//' comment
    starts nothing)."""
    out, i, n = [], 0, len(text)
    while i < n:
        if text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        else:
            out.append(text[i])
            i += 1
    return "".join(out)


def _body(src, fname):
    i = src.index("void %s()" % fname)
    j = src.find("\nvoid ", i + 1)
    return _strip_comments(src[i:j if j > 0 else len(src)])


def _ints(body):
    out = {}
    for name in ("n", "cmcc", "pncc", "p", "steps"):
        m = re.search(r"const int %s\s*=\s*(\d+)\s*;" % name, body)
        if m is None and name == "steps":  # test_no_proc_noise: int num_steps = 30;
            m = re.search(r"int num_steps\s*=\s*(\d+)\s*;", body)
        out[name] = int(m.group(1))
    return out


def _array(body, name, size):
    m = re.search(r"double %s\[[^\]]*\]\s*=\s*\{([^}]*)\}" % name, body, flags=re.S)
    vals = [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
    arr = np.zeros(size)
    arr[:len(vals)] = vals  # C zero-fills an initialiser shorter than the array
    return arr


def problem(src, fname):
    body = _body(src, fname)
    k = _ints(body)
    n, pncc, p, steps = k["n"], k["pncc"], k["p"], k["steps"]
    prob = {
        "d": n, "pncc": pncc, "cmcc": k["cmcc"], "p": p, "steps": steps, "B": None,
        "Phi": _array(body, "Phi", n * n).reshape(n, n),
        # no process noise: Gamma and beta are NULL pointers in the demo
        "Gamma": _array(body, "Gamma", n * pncc).reshape(n, pncc) if pncc else np.zeros((n, 0)),
        "H": _array(body, "H", p * n).reshape(p, n),
        "beta": _array(body, "beta", pncc) if pncc else np.zeros(0),
        "gamma": _array(body, "gamma", p),
        "A0": _array(body, "A0", n * n).reshape(n, n),
        "p0": _array(body, "p0", n),
        "b0": _array(body, "b0", n),
        "msmts": _array(body, "zs", steps * p).reshape(steps, p),
    }
    return prob


if __name__ == "__main__":
    oracle.build()
    src = open(os.path.join(oracle.REFERENCE_ROOT, "src", "cauchy_estimator.cpp")).read()
    for name, fname, seed in DEMOS:
        prob = problem(src, fname)
        n = make_golden.pack(name, prob, seed, print_basic_info=True)
        z = np.load(os.path.join(HERE, name + ".npz"))
        print(name, "updates", n, "terms", [int(z["u%d_Nt" % i]) for i in range(n)],
              "errors", [int(z["u%d_err" % i]) for i in range(n)])
