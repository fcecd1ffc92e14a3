"""Numpy restatement of tupan's SIA integrators -- TEST INFRASTRUCTURE ONLY
(parity checker for the device-resident SIA driver).

The recursion follows tupan/integrator/sia.py with copies for every split
and a concatenation for every join, exactly as the reference's particle
system does, and calls the oracle kernels for every pairwise sum, so a run
is bit-identical to the reference on its C backend (the Kepler solver of
two-body subsets calls libm, like the reference C):

* ``split`` / ``join``   sia.py:22-55 (stable slow/fast partition; a
                         subsystem of at most two particles is not split)
* ``drift`` / ``kick``   sia.py:58-81, :160-182 (Newtonian operators; the
                         kick sets the subsystem's own acceleration first)
* ``sf_kick``            sia.py:199-297 (mutual accelerations, Newtonian
                         branch only)
* ``_evolve``            SIAnn.dkd / SIAnn.kdk; FewBody.evolve
                         (fewbody.py:43-60) below three particles
* ``_bridge``            SIAnn.bridge_sf (sf_drift/sf_kick sequence)
* ``_recurse``           SIA.recurse (sia.py:1097-1123)
* ``sia_step``           SIA.do_step (sia.py:1034-1095) for one base step
* ``evolve``             Base.evolve_step loop (integrator/__init__.py:80-99)

Coefficient tables: sia.py:300-864 (the published splitting coefficients of
Yoshida 1990, Omelyan, Mryglod & Folk 2003, Blanes & Moan 2002 and Kahan &
Li 1997).  Every propagator is the palindrome that interleaves the second
coefficient list ("outer" operator) with the first ("inner" operator):
o0 i0 o1 i1 ... mirrored about its middle element.  For dkd and bridge_sf
the outer operator is the drift, for kdk the kick.

A state is a dict of float64 arrays m, e2, rx, ry, rz, vx, vy, vz, ax, ay,
az, tstep, time and int64 arrays nstep, id.  Post-Newtonian corrections are
not restated (the device driver is Newtonian only).
"""

import numpy as np

import oracle
from oracle.integrators import base_tstep, block_tstep

COEFS = {
    "sia21": ([1.0], [0.5]),
    "sia22": ([0.5], [0.1931833275037836, 0.6136333449924328]),
    "sia43": ([1.3512071919596575, -1.7024143839193150],
              [0.6756035959798288, -0.17560359597982877]),
    "sia44": ([0.7123418310626056, -0.21234183106260562],
              [0.1786178958448091, -0.06626458266981843, 0.7752933736500186]),
    "sia45": ([-0.0844296195070715, 0.354900057157426, 0.459059124699291],
              [0.2750081212332419, -0.1347950099106792, 0.35978688867743724]),
    "sia46": ([0.209515106613362, -0.143851773179818, 0.434336666566456],
              [0.0792036964311957, 0.353172906049774, -0.0420650803577195,
               0.21937695575349958]),
    "sia67": ([0.7845136104775573, 0.23557321335935813, -1.177679984178871,
               1.3151863206839112],
              [0.39225680523877865, 0.5100434119184577, -0.47105338540975644,
               0.06875316825252015]),
    "sia69": ([0.39103020330868477, 0.334037289611136, -0.7062272811875614,
               0.08187754964805945, 0.7985644772393624],
              [0.19551510165434238, 0.3625337464599104, -0.1860949957882127,
               -0.31217486576975095, 0.44022101344371095]),
}

FIELDS = ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz", "ax", "ay", "az",
          "tstep", "time", "nstep", "id")
POS = ("rx", "ry", "rz")
VEL = ("vx", "vy", "vz")
ACC = ("ax", "ay", "az")


def sequence(scheme):
    """[(is_outer, coefficient), ...] of one propagator of ``scheme``."""
    inner, outer = COEFS[scheme]
    fwd = []
    for k in range(len(outer)):
        fwd.append((True, outer[k]))
        if k < len(inner):
            fwd.append((False, inner[k]))
        if len(fwd) >= len(outer) + len(inner):
            break
    return fwd + fwd[-2::-1]


def parse(method):
    """'sia21h.dkd' -> ('sia21', 'h', 'dkd')"""
    head, kind = method.split(".")
    return head[:5], head[5], kind


def new_state(ps):
    n = len(ps["m"])
    st = {k: np.ascontiguousarray(ps[k], dtype=np.float64).copy()
          for k in ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    for k in ("ax", "ay", "az", "tstep", "time"):
        st[k] = np.zeros(n)
    st["nstep"] = np.zeros(n, dtype=np.int64)
    st["id"] = np.arange(n, dtype=np.int64)
    return st


def _n(ps):
    return len(ps["m"])


def _take(ps, sel):
    return {k: ps[k][sel].copy() for k in FIELDS}


def split(ps, cond):
    """sia.py:22-39"""
    if _n(ps) <= 2:
        return ps, _take(ps, np.zeros(_n(ps), dtype=bool))
    return _take(ps, cond), _take(ps, ~cond)


def join(slow, fast):
    """sia.py:42-55"""
    if not _n(fast):
        return slow
    if not _n(slow):
        return fast
    return {k: np.concatenate([slow[k], fast[k]]) for k in FIELDS}


def _set_acc(ips, jps):
    ips["ax"], ips["ay"], ips["az"] = oracle.run("acc_kernel", ips, jps)


def drift(ps, tau):
    """sia.py:58-67 (drift_n), fewbody.py:16-25"""
    for r, v in zip(POS, VEL):
        ps[r] += ps[v] * tau


def kick_n(ps, tau):
    """sia.py:70-79"""
    for v, a in zip(VEL, ACC):
        ps[v] += ps[a] * tau


def kick(ps, tau):
    """sia.py:173-182"""
    _set_acc(ps, ps)
    kick_n(ps, tau)


def fewbody(ps, tau):
    """FewBody.evolve (fewbody.py:43-60)."""
    n = _n(ps)
    if n == 0:
        return
    if n == 1:
        drift(ps, tau)
        return
    out = oracle.run("kepler_solver_kernel", ps, ps, {"dt": tau})
    for k, v in zip(POS + VEL, out):
        ps[k][...] = v


class Run:
    """One SIA integration: method flags, the global t_curr and the
    recursion of sia.py:1097-1123."""

    def __init__(self, method, eta):
        self.scheme, self.mode, self.kind = parse(method)
        if self.scheme not in COEFS or self.mode not in "sah" or \
                self.kind not in ("dkd", "kdk"):
            raise ValueError("unexpected method: %s" % method)
        self.eta = eta
        self.t_curr = 0.0
        self.seq = sequence(self.scheme)

    def _evolve(self, ps, tau):
        """SIAnn.dkd / SIAnn.kdk"""
        if _n(ps) <= 2:
            fewbody(ps, tau)
            return ps
        for outer, c in self.seq:
            is_drift = outer == (self.kind == "dkd")
            if is_drift:
                drift(ps, c * tau)
            else:
                kick(ps, c * tau)
        return ps

    def _bridge(self, slow, fast, tau):
        """SIAnn.bridge_sf: sf_drift for the outer coefficients, sf_kick
        for the inner ones."""
        for outer, c in self.seq:
            if outer:
                slow = self._evolve(slow, c * tau)
                fast = self._recurse(fast, c * tau)
            elif _n(slow) and _n(fast):
                _set_acc(slow, fast)
                _set_acc(fast, slow)
                kick_n(slow, c * tau)
                kick_n(fast, c * tau)
        return slow, fast

    def _recurse(self, ps, tau):
        if not _n(ps):
            return ps
        flag = -1
        if self.mode in "ah":
            flag = 1
            ps["tstep"], _ = oracle.run("tstep_kernel", ps, ps,
                                        {"eta": self.eta})
            if self.mode == "a":
                tau = block_tstep(np.abs(ps["tstep"]).min(), self.t_curr,
                                  tau)
        slow, fast = split(ps, np.abs(ps["tstep"]) > flag * abs(tau))
        slow, fast = self._bridge(slow, fast, tau)
        if _n(fast) == 0:
            self.t_curr += tau
        if _n(slow):
            slow["tstep"][...] = tau
            slow["time"] += tau
            slow["nstep"] += 1
        return join(slow, fast)

    def step(self, ps, t_end):
        """Base.evolve_step + SIA.do_step: one base step."""
        tau = base_tstep(self.t_curr, t_end, self.eta)
        return self._recurse(ps, tau)


def evolve(ps, method, eta, t_end, max_steps=None):
    """Steps until |t_curr| >= t_end (or max_steps); returns the final state
    (in the reference's final particle order) and the t_curr after each
    step."""
    run = Run(method, eta)
    st = new_state(ps)
    times = []
    while abs(run.t_curr) < t_end:
        st = run.step(st, t_end)
        times.append(run.t_curr)
        if max_steps is not None and len(times) >= max_steps:
            break
    return st, times
