"""Test infrastructure: the CPU oracle for the MCE step path.

Two checkers live here, and only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs may use them:

* ``Oracle`` — ``mce_oracle.cpp``, a serial C++ restatement of the reference's
  ``CauchyEstimator::step`` (include/cauchy_estimator.hpp:1211-1245), built
  into ``oracle/_build`` by :func:`build`.
* ``Reference`` — ``ref_harness.cpp`` compiled from the reference's own headers
  where they lie (only when the reference sources are present), built into
  ``oracle/_ref``.  Used to generate the golden fixtures and to pin the oracle.

Both expose the same stepping interface so tests can run either on a problem
dict from :mod:`cauchyfriendly_gb300.workloads`.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# Where the reference checkout lies (read only at build time, by build()).
REFERENCE_ROOT = os.environ.get("MCE_REFERENCE_ROOT", "/root/reference")
# build() copies the reference's headers here (git-ignored) so that the
# reference C++ can also be compiled on a host without the checkout.
REF_SRC = os.path.join(REF_OUT, "src")
ORACLE_SO = os.path.join(BUILD, "libmce_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _ptr(a, kind=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(kind)


def _refresh_reference_copy():
    """Copies the reference's include/ and its SWIG glue header into
    oracle/_ref/src (git-ignored), keeping their relative layout, when the
    checkout is present.  Returns the include directory to compile against,
    or None when neither the checkout nor a copy exists."""
    import shutil
    inc = os.path.join(REFERENCE_ROOT, "include")
    if os.path.isdir(inc):
        dst_inc = os.path.join(REF_SRC, "include")
        glue = os.path.join(REFERENCE_ROOT, "scripts", "swig", "cauchy", "pycauchy.hpp")
        dst_glue = os.path.join(REF_SRC, "scripts", "swig", "cauchy")
        os.makedirs(dst_glue, exist_ok=True)
        shutil.copytree(inc, dst_inc, dirs_exist_ok=True)
        if os.path.exists(glue):
            shutil.copy2(glue, dst_glue)
        # the reference's Python API, for the tests that run it over the drop-in
        api = os.path.join(REFERENCE_ROOT, "scripts", "swig", "cauchy", "cauchy_estimator.py")
        if os.path.exists(api):
            shutil.copy2(api, dst_glue)
    own = os.path.join(REF_SRC, "include")
    return own if os.path.isdir(own) else None


def reference_python_api(pycauchy_module, name="reference_cauchy_estimator"):
    """The reference's Python API (scripts/swig/cauchy/cauchy_estimator.py,
    from the copy in oracle/_ref/src, unmodified) imported with ``pycauchy``
    bound to pycauchy_module and a stand-in for matplotlib (plotting is not
    used).  None when no copy exists."""
    import importlib.util
    import sys
    import types
    path = os.path.join(REF_SRC, "scripts", "swig", "cauchy", "cauchy_estimator.py")
    if not os.path.exists(path):
        return None
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    saved = sys.modules.get("pycauchy")
    sys.modules["pycauchy"] = pycauchy_module
    try:
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        if saved is None:
            sys.modules.pop("pycauchy", None)
        else:
            sys.modules["pycauchy"] = saved
    return mod


def host_cpus_pow2():
    """The largest power of two <= the host's core count (the reference's
    threaded term reduction and sort merges need a power of two)."""
    n = 1
    while n * 2 <= (os.cpu_count() or 1):
        n *= 2
    return n


def build(force=False, with_reference=True, verbose=False):
    """Compiles the oracle (always) and the reference harnesses (when the
    reference headers are present, as a checkout or as the copy in
    oracle/_ref/src).  -ffp-contract=off keeps a*b+c unfused on every host so
    results match across x86 and aarch64."""
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    src = os.path.join(HERE, "mce_oracle.cpp")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        jobs.append(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", src,
                     "-o", ORACLE_SO, "-lpthread"])
    inc = _refresh_reference_copy() if with_reference else None
    if inc:
        os.makedirs(REF_OUT, exist_ok=True)
        glue_dir = os.path.join(REF_SRC, "scripts", "swig", "cauchy")
        ncpu = host_cpus_pow2()
        targets = [("libmce_ref_serial.so", "ref_harness.cpp", 1), ("libmce_ref_threaded.so", "ref_harness.cpp", ncpu)]
        if os.path.exists(os.path.join(glue_dir, "pycauchy.hpp")):
            targets.append(("libmce_ref_pycauchy.so", "ref_pycauchy.cpp", 1))
        for name, cpp, n in targets:
            out = os.path.join(REF_OUT, name)
            hsrc = os.path.join(HERE, cpp)
            if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(hsrc):
                jobs.append(["g++", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I" + inc,
                             "-I" + glue_dir, "-DHARNESS_NUM_CPUS=%d" % n, hsrc, "-o", out, "-lpthread"])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(j), out.decode()))
        if verbose:
            print(" ".join(j))


def reference_available():
    """True when the reference harness is built for this host and loads (a
    copy built on another architecture does not)."""
    path = os.path.join(REF_OUT, "libmce_ref_serial.so")
    if not os.path.exists(path):
        return False
    try:
        ctypes.CDLL(path)
    except OSError:
        return False
    return True


_libc = ctypes.CDLL(None)


def draw_reference_constants(seed, d, max_shape, num_cpus=8):
    """Reproduces the reference constructor's libc rand() draws after
    srand(seed): root_point[i] = 1 + U(0,1] (include/cauchy_estimator.hpp:127-128)
    then num_cpus DCE helpers each draw b_pert[i] = 2 U(0,1] - 1
    (include/cell_enumeration.hpp:467-470); helper 0's b_pert is returned."""
    _libc.srand(ctypes.c_uint(seed))
    rmax = 2147483647.0

    def u():
        return (float(_libc.rand()) + 1.0) / (rmax + 1.0)

    root = np.array([1.0 + u() for _ in range(d)])
    bpert = None
    for h in range(num_cpus):
        bp = np.array([2.0 * u() - 1.0 for _ in range(max_shape)])
        if h == 0:
            bpert = bp
    return root, bpert


def max_shape_of(prob):
    d, pncc = prob["d"], prob["pncc"]
    return (prob["steps"] - 1) * pncc + d if d > 1 else d + pncc


class _Lib:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        L = self.lib
        f = lambda n: getattr(L, prefix + n)
        f("step").restype = ctypes.c_int
        f("step").argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp, _dp, ctypes.c_double, _dp, _dp]
        f("destroy").argtypes = [ctypes.c_void_p]
        f("num_terms").argtypes = [ctypes.c_void_p]
        f("shape_range").argtypes = [ctypes.c_void_p]
        f("terms_per_shape").argtypes = [ctypes.c_void_p, _ip]
        f("get_moments").argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        f("total_cells").restype = ctypes.c_longlong
        f("total_cells").argtypes = [ctypes.c_void_p]
        f("dump_terms").argtypes = [ctypes.c_void_p, _ip, _dp, _dp, _dp, _ip, _ip, _dp]

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)


class _EstimatorBase:
    """Common stepping/readout over the oracle or the reference harness."""

    def __init__(self, lib, handle, prob):
        self._l = lib
        self.h = handle
        self.prob = prob
        self.d = prob["d"]

    def step(self, k, sub=0):
        """Feeds measurement ``sub`` of step ``k``; returns the error bitmask."""
        prob = self.prob
        Phi = np.ascontiguousarray(prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][k], dtype=np.float64)
        Gamma = np.ascontiguousarray(prob["Gamma"], dtype=np.float64)
        beta = np.ascontiguousarray(prob["beta"], dtype=np.float64)
        H = np.ascontiguousarray(prob["H"][sub], dtype=np.float64)
        B = None if prob.get("B") is None else np.ascontiguousarray(prob["B"], dtype=np.float64)
        u = None
        if B is not None:
            u = np.ascontiguousarray(prob["u"][k], dtype=np.float64)
        z = float(prob["msmts"][k, sub])
        return self._l.fn("step")(self.h, z, _ptr(Phi), _ptr(Gamma), _ptr(beta), _ptr(H),
                                  float(prob["gamma"][sub]), _ptr(B), _ptr(u))

    def moments(self):
        d = self.d
        fz = np.zeros(2); mean = np.zeros(2 * d); cov = np.zeros(2 * d * d)
        rfz = np.zeros(2); rmean = np.zeros(2 * d); rcov = np.zeros(2 * d * d)
        gs = np.zeros(1)
        self._l.fn("get_moments")(self.h, _ptr(fz), _ptr(mean), _ptr(cov), _ptr(rfz), _ptr(rmean),
                                  _ptr(rcov), _ptr(gs))
        c = lambda a: a[0::2] + 1j * a[1::2]
        return {"fz": complex(fz[0], fz[1]), "mean": c(mean), "cov": c(cov).reshape(d, d),
                "raw_fz": complex(rfz[0], rfz[1]), "raw_mean": c(rmean), "raw_cov": c(rcov).reshape(d, d),
                "gscale": float(gs[0])}

    def num_terms(self):
        return int(self._l.fn("num_terms")(self.h))

    def terms_per_shape(self):
        n = int(self._l.fn("shape_range")(self.h))
        out = np.zeros(n, dtype=np.int32)
        self._l.fn("terms_per_shape")(self.h, _ptr(out, _ip))
        return out

    def dump_terms(self, max_shape):
        nt = self.num_terms()
        tc = int(self._l.fn("total_cells")(self.h))
        d = self.d
        shape = np.zeros(nt, dtype=np.int32)
        A = np.zeros(nt * max_shape * d)
        p = np.zeros(nt * max_shape)
        b = np.zeros(nt * d)
        cells = np.zeros(nt, dtype=np.int32)
        keys = np.zeros(max(tc, 1), dtype=np.int32)
        g = np.zeros(2 * max(tc, 1))
        self._l.fn("dump_terms")(self.h, _ptr(shape, _ip), _ptr(A), _ptr(p), _ptr(b), _ptr(cells, _ip),
                                 _ptr(keys, _ip), _ptr(g))
        return {"shape": shape, "A": A.reshape(nt, max_shape, d), "p": p.reshape(nt, max_shape),
                "b": b.reshape(nt, d), "cells": cells, "keys": keys[:tc],
                "g": (g[0::2] + 1j * g[1::2])[:tc]}

    def close(self):
        if self.h:
            self._l.fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_oracle_lib = None
_ref_libs = {}


def _load_oracle():
    global _oracle_lib
    if _oracle_lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_reference=False)
        lib = _Lib(ORACLE_SO, "orc_")
        lib.lib.orc_create.restype = ctypes.c_void_p
        lib.lib.orc_create.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, _dp, _dp]
        lib.lib.orc_post_mu_terms.restype = ctypes.c_longlong
        lib.lib.orc_post_mu_terms.argtypes = [ctypes.c_void_p]
        lib.lib.orc_reset.argtypes = [ctypes.c_void_p]
        lib.lib.orc_reinit.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        lib.lib.orc_set_master_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.lib.orc_errors.argtypes = [ctypes.c_void_p]
        _oracle_lib = lib
    return _oracle_lib


def _load_ref(threaded=False):
    name = "libmce_ref_threaded.so" if threaded else "libmce_ref_serial.so"
    if name not in _ref_libs:
        path = os.path.join(REF_OUT, name)
        if not os.path.exists(path):
            raise FileNotFoundError(path + " (reference harness not built; needs the reference sources)")
        lib = _Lib(path, "ref_")
        lib.lib.ref_create.restype = ctypes.c_void_p
        lib.lib.ref_create.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_uint]
        lib.lib.ref_get_constants.argtypes = [ctypes.c_void_p, _dp, _dp, _ip]
        lib.lib.ref_last_step_seconds.restype = ctypes.c_double
        lib.lib.ref_last_step_seconds.argtypes = [ctypes.c_void_p]
        _ref_libs[name] = lib
    return _ref_libs[name]


def _arr(x):
    return np.ascontiguousarray(x, dtype=np.float64)


class Oracle(_EstimatorBase):
    def __init__(self, prob, root_point, b_pert):
        lib = _load_oracle()
        A0, p0, b0 = _arr(prob["A0"]), _arr(prob["p0"]), _arr(prob["b0"])
        rp, bp = _arr(root_point), _arr(b_pert)
        h = lib.lib.orc_create(_ptr(A0), _ptr(p0), _ptr(b0), prob["steps"], prob["d"], prob["cmcc"],
                               prob["pncc"], prob["p"], _ptr(rp), _ptr(bp))
        super().__init__(lib, h, prob)

    def post_mu_terms(self):
        return int(self._l.lib.orc_post_mu_terms(self.h))

    def step_with(self, msmt, Phi, Gamma, beta, H, gamma):
        """One update with explicit model arrays (window-manager use)."""
        a = lambda x: np.ascontiguousarray(x, dtype=np.float64)
        Phi, Gamma, beta, H = a(Phi), a(Gamma), a(beta), a(H)
        return self._l.fn("step")(self.h, float(msmt), _ptr(Phi), _ptr(Gamma), _ptr(beta), _ptr(H), float(gamma),
                                  None, None)

    def reset(self):
        self._l.lib.orc_reset(self.h)

    def reinit(self, A0, p0, b0):
        a = lambda x: np.ascontiguousarray(x, dtype=np.float64)
        A0, p0, b0 = a(A0), a(p0), a(b0)
        self._l.lib.orc_reinit(self.h, _ptr(A0), _ptr(p0), _ptr(b0))

    def set_master_step(self, ms):
        self._l.lib.orc_set_master_step(self.h, int(ms))

    def errors(self):
        return int(self._l.lib.orc_errors(self.h))

    def set_print_basic_info(self, on):
        """The constructor's print_basic_info: post-FTR moments are reported."""
        self._l.lib.orc_set_print_basic_info.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self._l.lib.orc_set_print_basic_info(self.h, int(bool(on)))

    def shift_cf_by_bias(self, bias):
        b = _arr(bias)
        self._l.lib.orc_shift_cf_by_bias.argtypes = [ctypes.c_void_p, _dp]
        self._l.lib.orc_shift_cf_by_bias(self.h, _ptr(b))

    def deterministic_time_prop(self, Phi, B=None, u=None):
        f = self._l.lib.orc_deterministic_time_prop
        f.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        Phi = _arr(Phi)
        B = None if B is None else _arr(B)
        u = None if u is None else _arr(u)
        f(self.h, _ptr(Phi), _ptr(B), _ptr(u))

    def finalize_extended_moments(self, x_bar):
        x = _arr(x_bar).copy()
        self._l.lib.orc_finalize_extended_moments.argtypes = [ctypes.c_void_p, _dp]
        self._l.lib.orc_finalize_extended_moments(self.h, _ptr(x))
        return x

    def cpdf_2d_grid(self, i1, i2, bar_nu, gx, gy, reset_cache=False, max_points=200000):
        """Marginal 2-D pdf on the grid gx = (low, high, res) x gy (the
        reference's CauchyCPDFGridDispatcher2D); returns (x, y, z)."""
        f = self._l.lib.orc_cpdf_2d_grid
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp] + [ctypes.c_double] * 6 + \
            [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        nu = _arr(bar_nu)
        xs, ys, zs = np.zeros(max_points), np.zeros(max_points), np.zeros(max_points)
        n = f(self.h, int(i1), int(i2), _ptr(nu), *[float(v) for v in gx], *[float(v) for v in gy],
              int(bool(reset_cache)), max_points, _ptr(xs), _ptr(ys), _ptr(zs))
        if n < 0:
            raise RuntimeError("orc_cpdf_2d_grid returned %d" % n)
        return xs[:n].copy(), ys[:n].copy(), zs[:n].copy()

    def cpdf_1d_grid(self, marg, bar_nu, low, high, res, max_points=100000):
        """Marginal 1-D pdf on the grid low..high step res (the reference's
        CauchyCPDFGridDispatcher1D); returns (x, y) or raises with the status."""
        f = self._l.lib.orc_cpdf_1d_grid
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int, _dp, _dp]
        nu = _arr(bar_nu)
        xs, ys = np.zeros(max_points), np.zeros(max_points)
        n = f(self.h, int(marg), _ptr(nu), float(low), float(high), float(res), max_points, _ptr(xs), _ptr(ys))
        if n < 0:
            raise RuntimeError("orc_cpdf_1d_grid returned %d" % n)
        return xs[:n].copy(), ys[:n].copy()

    def cpdf_nd(self, x, reduce=True):
        """The N-D conditional pdf at the point x (complex; the reference's
        PointWiseNDimCauchyCPDF::evaluate_cpdf).  reduce=False keeps every
        lowered child apart (no term reduction between the lowerings)."""
        return _cpdf_nd_call(self._l.lib.orc_cpdf_nd, self.h, x, "orc_cpdf_nd", 1 if reduce else 0)

    def cpdf_marginal(self, xm, idx, nu_bar, reduce=True):
        """The marginal pdf of the states idx (ascending, fewer than d) at xm
        (complex; the reference's PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf),
        the last lookups at nu_bar (d - len(idx) values)."""
        f = self._l.lib.orc_cpdf_marginal
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, _dp, _ip, ctypes.c_int, _dp, _dp, ctypes.c_int]
        xx, nb = _arr(xm), _arr(nu_bar)
        ii = np.ascontiguousarray(np.asarray(idx, dtype=np.int32))
        out = np.zeros(2)
        st = f(self.h, _ptr(xx), _ptr(ii, _ip), len(ii), _ptr(nb), _ptr(out), 1 if reduce else 0)
        if st < 0:
            raise RuntimeError("orc_cpdf_marginal returned %d" % st)
        return complex(out[0], out[1])


class OracleSlot:
    """A window slot of n_mgr oracle estimators with the batch interface the
    window manager drives (cauchyfriendly_gb300.windows)."""

    def __init__(self, A0, p0, b0, steps, d, cmcc, pncc, p, consts):
        self.ests = []
        for m in range(A0.shape[0]):
            prob = {"A0": A0[m], "p0": p0[m], "b0": b0[m], "steps": steps, "d": d, "cmcc": cmcc, "pncc": pncc,
                    "p": p}
            self.ests.append(Oracle(prob, *consts[m]))

    def step(self, z, Phi, Gamma, beta, H, gamma):
        return np.array([e.step_with(z[m], Phi[m], Gamma[m], beta[m], H[m], gamma[m])
                         for m, e in enumerate(self.ests)], dtype=np.int32)

    def moments(self, i):
        return self.ests[i].moments()

    def errors(self, i):
        return self.ests[i].errors()

    def num_terms(self, i):
        return self.ests[i].num_terms()

    def reset(self):
        for e in self.ests:
            e.reset()

    def reinit(self, i, A0, p0, b0):
        self.ests[i].reinit(A0, p0, b0)

    def set_master_step(self, ms):
        for e in self.ests:
            e.set_master_step(ms)

    def post_mu_terms(self):
        return sum(e.post_mu_terms() for e in self.ests)

    def close(self):
        for e in self.ests:
            e.close()


class Reference(_EstimatorBase):
    def __init__(self, prob, seed=0, threaded=False):
        lib = _load_ref(threaded)
        A0, p0, b0 = _arr(prob["A0"]), _arr(prob["p0"]), _arr(prob["b0"])
        h = lib.lib.ref_create(_ptr(A0), _ptr(p0), _ptr(b0), prob["steps"], prob["d"], prob["cmcc"],
                               prob["pncc"], prob["p"], seed)
        super().__init__(lib, h, prob)

    def constants(self):
        ms = max_shape_of(self.prob)
        rp = np.zeros(self.d)
        bp = np.zeros(ms)
        n = ctypes.c_int(0)
        self._l.lib.ref_get_constants(self.h, _ptr(rp), _ptr(bp), ctypes.byref(n))
        return rp, bp

    def last_step_seconds(self):
        return float(self._l.lib.ref_last_step_seconds(self.h))

    def set_print_basic_info(self, on):
        """The constructor's print_basic_info (the reference also prints its progress)."""
        self._l.lib.ref_set_print_basic_info.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self._l.lib.ref_set_print_basic_info(self.h, int(bool(on)))

    def shift_cf_by_bias(self, bias):
        b = _arr(bias)
        self._l.lib.ref_shift_cf_by_bias.argtypes = [ctypes.c_void_p, _dp]
        self._l.lib.ref_shift_cf_by_bias(self.h, _ptr(b))

    def deterministic_time_prop(self, Phi, B=None, u=None):
        f = self._l.lib.ref_deterministic_time_prop
        f.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        Phi = _arr(Phi)
        B = None if B is None else _arr(B)
        u = None if u is None else _arr(u)
        f(self.h, _ptr(Phi), _ptr(B), _ptr(u))

    def finalize_extended_moments(self, x_bar):
        x = _arr(x_bar).copy()
        self._l.lib.ref_finalize_extended_moments.argtypes = [ctypes.c_void_p, _dp]
        self._l.lib.ref_finalize_extended_moments(self.h, _ptr(x))
        return x

    def cpdf_2d_grid(self, i1, i2, gx, gy, reset_cache=False, max_points=200000):
        """The reference's own marginal 2-D pdf grid; returns (x, y, z, bar_nu)."""
        f = self._l.lib.ref_cpdf_2d_grid
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + \
            [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp]
        xs, ys, zs, nu = np.zeros(max_points), np.zeros(max_points), np.zeros(max_points), np.zeros(self.d)
        n = f(self.h, int(i1), int(i2), *[float(v) for v in gx], *[float(v) for v in gy], int(bool(reset_cache)),
              max_points, _ptr(xs), _ptr(ys), _ptr(zs), _ptr(nu))
        if n < 0:
            raise RuntimeError("ref_cpdf_2d_grid returned %d" % n)
        return xs[:n].copy(), ys[:n].copy(), zs[:n].copy(), nu

    def cpdf_nd(self, x):
        """The reference's own PointWiseNDimCauchyCPDF::evaluate_cpdf at x."""
        return _cpdf_nd_call(self._l.lib.ref_cpdf_nd, self.h, x, "ref_cpdf_nd", None)

    def cpdf_marginal(self, xm, idx, seed):
        """The reference's own evaluate_marginal_cpdf of the states idx at xm
        after srand(seed); returns (value, nu_bar it drew)."""
        f = self._l.lib.ref_cpdf_marginal
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, _dp, _ip, ctypes.c_int, ctypes.c_uint, _dp, _dp]
        xx = _arr(xm)
        ii = np.ascontiguousarray(np.asarray(idx, dtype=np.int32))
        nb = np.zeros(self.d - len(ii))
        out = np.zeros(2)
        st = f(self.h, _ptr(xx), _ptr(ii, _ip), len(ii), int(seed), _ptr(nb), _ptr(out))
        if st < 0:
            raise RuntimeError("ref_cpdf_marginal returned %d" % st)
        return complex(out[0], out[1]), nb

    def cpdf_1d_grid(self, marg, low, high, res, max_points=100000):
        """The reference's own marginal 1-D pdf grid; returns (x, y, bar_nu)."""
        f = self._l.lib.ref_cpdf_1d_grid
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int, _dp, _dp, _dp]
        xs, ys, nu = np.zeros(max_points), np.zeros(max_points), np.zeros(self.d)
        n = f(self.h, int(marg), float(low), float(high), float(res), max_points, _ptr(xs), _ptr(ys), _ptr(nu))
        if n < 0:
            raise RuntimeError("ref_cpdf_1d_grid returned %d" % n)
        return xs[:n].copy(), ys[:n].copy(), nu



def _cpdf_nd_call(f, h, x, name, reduce):
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, _dp, _dp] + ([] if reduce is None else [ctypes.c_int])
    xx = _arr(x)
    out = np.zeros(2)
    st = f(h, _ptr(xx), _ptr(out)) if reduce is None else f(h, _ptr(xx), _ptr(out), reduce)
    if st < 0:
        raise RuntimeError("%s returned %d" % (name, st))
    return complex(out[0], out[1])


def _unpack_rel_moments(mom):
    return {"fz": complex(mom[0], mom[1]), "mean": mom[2:6:2] + 1j * mom[3:6:2],
            "cov": (mom[6:14:2] + 1j * mom[7:14:2]).reshape(2, 2)}


def oracle_rel2d(prim, sec, Trel, bar_nu_full, gx, gy, full_solve=False, with_term_approx=True,
                 term_approx_eps=1e-8, center=True, max_points=200000, pair_stride=1, pair_offset=0):
    """Relative-then-transformed system of two oracle estimators
    (rel = sec - prim, projected by the 2 x d Trel): its moments, pair counts
    and 2-D pdf on the grid gx = (low, high, step) x gy, offset by the
    relative mean when center (as pycauchy_single_step_eval_2d_rsys_cpdf).
    pair_stride > 1 takes only the pairs whose index is pair_offset modulo
    pair_stride (a timing sample)."""
    lib = prim._l.lib
    f = lib.orc_rel2d_create
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_double, _dp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int),
                  ctypes.c_longlong, ctypes.c_longlong]
    T, nu = _arr(Trel), _arr(bar_nu_full)
    mom = np.zeros(14)
    counts = (ctypes.c_longlong * 2)()
    st = ctypes.c_int(0)
    r = f(prim.h, sec.h, _ptr(T), _ptr(nu), int(bool(full_solve)), 1, int(bool(with_term_approx)),
          float(term_approx_eps), _ptr(mom), counts, ctypes.byref(st), int(pair_stride), int(pair_offset))
    if not r:
        raise RuntimeError("orc_rel2d_create status %d" % st.value)
    try:
        out = _unpack_rel_moments(mom)
        out["pairs"], out["approxed_out"] = int(counts[0]), int(counts[1])
        g = lib.orc_rel2d_grid
        g.restype = ctypes.c_int
        g.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 8 + [ctypes.c_int, _dp, _dp, _dp]
        ox, oy = (mom[2], mom[4]) if center else (0.0, 0.0)
        xs, ys, zs = np.zeros(max_points), np.zeros(max_points), np.zeros(max_points)
        n = g(r, gx[0] + ox, gx[1] + ox, float(gx[2]), gy[0] + oy, gy[1] + oy, float(gy[2]),
              float(prim.moments()["fz"].real), float(sec.moments()["fz"].real), max_points, _ptr(xs), _ptr(ys),
              _ptr(zs))
        if n < 0:
            raise RuntimeError("orc_rel2d_grid returned %d" % n)
        out["x"], out["y"], out["z"] = xs[:n].copy(), ys[:n].copy(), zs[:n].copy()
    finally:
        lib.orc_rel2d_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_rel2d_destroy(r)
    return out


def reference_rel2d(prim, sec, Trel, bar_seed, gx, gy, full_solve=False, with_term_approx=True,
                    term_approx_eps=1e-8, center=True, max_points=200000):
    """The reference's own relative-then-transformed system of two reference
    estimators; the same dictionary as oracle_rel2d plus "bar_nu_full", the
    point the reference drew after srand(bar_seed)."""
    lib = prim._l.lib
    f = lib.ref_rel2d
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _dp, ctypes.c_uint, ctypes.c_int, ctypes.c_int,
                  ctypes.c_double] + [ctypes.c_double] * 6 + [ctypes.c_int, ctypes.c_int, _dp, _dp,
                                                              ctypes.POINTER(ctypes.c_longlong), _dp, _dp, _dp]
    T = _arr(Trel)
    nu, mom = np.zeros(prim.d), np.zeros(14)
    counts = (ctypes.c_longlong * 2)()
    xs, ys, zs = np.zeros(max_points), np.zeros(max_points), np.zeros(max_points)
    n = f(prim.h, sec.h, _ptr(T), int(bar_seed), int(bool(full_solve)), int(bool(with_term_approx)),
          float(term_approx_eps), *[float(v) for v in gx[:2]], float(gx[2]), *[float(v) for v in gy[:2]],
          float(gy[2]), int(bool(center)), max_points, _ptr(nu), _ptr(mom), counts, _ptr(xs), _ptr(ys), _ptr(zs))
    if n < 0:
        raise RuntimeError("ref_rel2d returned %d" % n)
    out = _unpack_rel_moments(mom)
    out["pairs"], out["approxed_out"] = int(counts[0]), int(counts[1])
    out["x"], out["y"], out["z"] = xs[:n].copy(), ys[:n].copy(), zs[:n].copy()
    out["bar_nu_full"] = nu
    return out

def run(est, prob, record_terms_upto=0):
    """Steps ``est`` through the whole problem; returns per-measurement records."""
    recs = []
    ms = max_shape_of(prob)
    total = prob["steps"] * prob["p"]
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            err = est.step(k, s)
            n += 1
            rec = est.moments()
            rec["err"] = int(err)
            rec["Nt"] = est.num_terms()
            rec["tps"] = est.terms_per_shape()
            if n < total and rec["Nt"] <= record_terms_upto:
                rec["terms"] = est.dump_terms(ms)
            recs.append(rec)
    return recs


def run_oracle_batch(probs, constants, threads=None):
    """Runs independent problems on a thread pool (each estimator serial).
    Returns (total post-MU term count, wall seconds)."""
    import time
    threads = threads or (os.cpu_count() or 1)

    def one(i):
        est = Oracle(probs[i], *constants[i])
        for k in range(probs[i]["steps"]):
            for s in range(probs[i]["p"]):
                est.step(k, s)
        n = est.post_mu_terms()
        est.close()
        return n

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        counts = list(ex.map(one, range(len(probs))))
    return int(sum(counts)), time.perf_counter() - t0


# ---- the reference's own C++ over a process pool (CPU baseline) ------------
# One estimator per task, the serial build in every worker: the reference's
# estimator keeps process-wide state (function pointers, flags, the harness's
# raw-moment hook), so independent estimators run in separate processes, as the
# reference's own window manager runs its windows.

_POOL_PROBS = None
_POOL_SEEDS = None


def _pool_init(probs, seeds):
    global _POOL_PROBS, _POOL_SEEDS
    _POOL_PROBS, _POOL_SEEDS = probs, seeds
    # the reference prints warnings on stdout; keep the caller's stdout clean
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)


def _pool_run(i):
    prob = _POOL_PROBS[i]
    est = Reference(prob, seed=_POOL_SEEDS[i])
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            est.step(k, s)
    est.close()
    return 1


class ReferencePool:
    """The reference's C++ (oracle/_ref, serial build) stepping independent
    estimators in `workers` processes (spawned).  run(indices) steps every
    listed estimator through its whole history and returns the wall seconds
    (the post-MU term count of the same work comes from the oracle port,
    which the tests hold equal to the reference's)."""

    def __init__(self, probs, seeds, workers=None):
        import multiprocessing as mp
        self.workers = workers or (os.cpu_count() or 1)
        self.probs = probs
        self.pool = mp.get_context("spawn").Pool(self.workers, initializer=_pool_init, initargs=(probs, seeds))

    def run(self, indices=None):
        import time
        idx = list(range(len(self.probs))) if indices is None else list(indices)
        # largest first (term counts grow about 3x per step), handed out one by one
        idx.sort(key=lambda i: -self.probs[i]["steps"] * self.probs[i]["p"])
        t0 = time.perf_counter()
        done = sum(self.pool.imap_unordered(_pool_run, idx, chunksize=1))
        assert done == len(idx)
        return time.perf_counter() - t0

    def close(self):
        self.pool.terminate()
        self.pool.join()
