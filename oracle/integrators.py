"""Numpy restatement of tupan's Hermite and Sakura integrators -- TEST
INFRASTRUCTURE ONLY (parity checker for the device-resident drivers).

Each function follows the reference statement by statement, with numpy fp64
elementwise arithmetic in the same order, and calls the oracle kernels for
the pairwise sums, so a run is bit-identical to the reference integrator on
the reference's C backend:

* ``block_tstep``   tupan/integrator/__init__.py:59-78 (get_min_block_tstep)
* ``base_tstep``    tupan/integrator/__init__.py:48-57 (get_base_tstep)
* ``hermite_step``  tupan/integrator/hermite.py:20-283 (H2/H4/H6/H8 epredict,
                    ecorrect, epec) and :390-410 (Hermite.do_step)
* ``sakura_step``   tupan/integrator/sakura.py:22-50, :100-117 (asakura step)
* ``evolve``        tupan/simulation.py:187-198 loop over evolve_step
                    (tupan/integrator/__init__.py:80-99)
* ``nreg_evolve``   tupan/integrator/nreg.py:22-170 (nreg_x, nreg_v,
                    anreg_step, nreg_step, NREG.initialize and do_step)
* ``pairwise_sum``  numpy's summation order for float64 arrays (the
                    reference's .sum() calls), restated for the device

A state is a dict of float64 arrays m, rx, ry, rz, e2, vx, vy, vz.
"""

import math
import sys

import numpy as np

import oracle

POS = ("rx", "ry", "rz")
VEL = ("vx", "vy", "vz")


def _kern(name, ips, jps=None, scal=None):
    return oracle.run(name, ips, jps if jps is not None else ips, scal)


def base_tstep(t_curr, t_end, eta):
    """tupan/integrator/__init__.py:48-57"""
    dt = min(abs(t_end) - abs(t_curr), abs(eta))
    dt = max(dt, abs(t_end) * (2 * sys.float_info.epsilon))
    return math.copysign(dt, eta)


def block_tstep(min_ts, t_curr, tau):
    """tupan/integrator/__init__.py:59-78 for a given min |tstep|."""
    power = int(np.log2(min_ts) - 1)
    min_bts = 2.0 ** power
    t_next = t_curr + min_bts
    while t_next % min_bts != 0:
        min_bts /= 2
    min_bts = math.copysign(min_bts, tau)
    if abs(min_bts) > abs(tau):
        min_bts = tau
    return min_bts


def forces(order, ps):
    """set_acc / set_acc_jerk / set_snap_crackle as each Hn.epredict and
    ecorrect call them (hermite.py:30, :80-81, :132-133, :206-207)."""
    f = {}
    if order == 2:
        f["ax"], f["ay"], f["az"] = _kern("acc_kernel", ps)
        return f
    out = _kern("acc_jerk_kernel", ps)
    for k, v in zip(("ax", "ay", "az", "jx", "jy", "jz"), out):
        f[k] = v
    if order >= 6:
        q = dict(ps)
        q.update(f)
        out = _kern("snap_crackle_kernel", q)
        for k, v in zip(("sx", "sy", "sz", "cx", "cy", "cz"), out):
            f[k] = v
    return f


def predict(order, ps, f0, tau):
    """Hn.epredict position/velocity updates (hermite.py:33-38, :83-88,
    :136-157, :210-235); ps is updated in place from the copy's values."""
    for c, (r, v) in enumerate(zip(POS, VEL)):
        a = f0["a" + "xyz"[c]]
        if order == 2:
            ps[r] = ps[r] + (a * tau / 2 + ps[v]) * tau
            ps[v] = ps[v] + a * tau
            continue
        j = f0["j" + "xyz"[c]]
        if order == 4:
            ps[r] = ps[r] + ((j * tau / 3 + a) * tau / 2 + ps[v]) * tau
            ps[v] = ps[v] + (j * tau / 2 + a) * tau
            continue
        s = f0["s" + "xyz"[c]]
        if order == 6:
            ps[r] = ps[r] + (((s * tau / 4 + j) * tau / 3 + a) * tau / 2
                             + ps[v]) * tau
            ps[v] = ps[v] + ((s * tau / 3 + j) * tau / 2 + a) * tau
            continue
        cr = f0["c" + "xyz"[c]]
        ps[r] = ps[r] + ((((cr * tau / 5 + s) * tau / 4 + j) * tau / 3 + a)
                         * tau / 2 + ps[v]) * tau
        ps[v] = ps[v] + (((cr * tau / 4 + s) * tau / 3 + j) * tau / 2
                         + a) * tau


def correct(order, ps1, ps0, f0, f1, tau):
    """Hn.ecorrect (hermite.py:46-57, :96-119, :162-195, :238-283).
    Velocities first, then positions from the corrected velocities."""
    for c, (r, v) in enumerate(zip(POS, VEL)):
        x = "xyz"[c]
        a0, a1 = f0["a" + x], f1["a" + x]
        if order == 2:
            ps1[v] = ((a0 + a1) * tau / 2 + ps0[v])
            ps1[r] = ((ps0[v] + ps1[v]) * tau / 2 + ps0[r])
            continue
        j0, j1 = f0["j" + x], f1["j" + x]
        if order == 4:
            ps1[v] = (((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + ps0[v])
            ps1[r] = (((a0 - a1) * tau / 6 + (ps0[v] + ps1[v])) * tau / 2
                      + ps0[r])
            continue
        s0, s1 = f0["s" + x], f1["s" + x]
        if order == 6:
            ps1[v] = ((((s0 + s1) * tau / 12 + (j0 - j1)) * tau / 5
                       + (a0 + a1)) * tau / 2 + ps0[v])
            ps1[r] = ((((j0 + j1) * tau / 12 + (a0 - a1)) * tau / 5
                       + (ps0[v] + ps1[v])) * tau / 2 + ps0[r])
            continue
        c0, c1 = f0["c" + x], f1["c" + x]
        ps1[v] = (((((c0 - c1) * tau / 20 + (s0 + s1)) * tau / 3
                    + 3 * (j0 - j1)) * tau / 14 + (a0 + a1)) * tau / 2
                  + ps0[v])
        ps1[r] = (((((s0 - s1) * tau / 20 + (j0 + j1)) * tau / 3
                    + 3 * (a0 - a1)) * tau / 14 + (ps0[v] + ps1[v])) * tau / 2
                  + ps0[r])


def hermite_step(ps, t_curr, tau, eta, order, adaptive):
    """Hermite.do_step (hermite.py:390-410) with epec(2, ...) (:60-67).
    Returns the step taken; ps is advanced in place."""
    if adaptive:
        dt_a, dt_b = _kern("tstep_kernel", ps, None, {"eta": eta})
        tau = block_tstep(np.abs(dt_a).min(), t_curr, tau)
    ps0 = {k: v.copy() for k, v in ps.items()}
    f0 = forces(order, ps0)
    predict(order, ps, f0, tau)
    for _ in range(2):
        f1 = forces(order, ps)
        correct(order, ps, ps0, f0, f1, tau)
    return tau


def sakura_step(ps, tau):
    """sakura.py:22-50"""
    for r, v in zip(POS, VEL):
        ps[r] = ps[r] + ps[v] * tau / 2
    for flag in (-1, 1):
        d = _kern("sakura_kernel", ps, None, {"dt": tau / 2, "flag": flag})
        for k, dv in zip(POS + VEL, d):
            ps[k] = ps[k] + dv
    for r, v in zip(POS, VEL):
        ps[r] = ps[r] + ps[v] * tau / 2


def sakura_tstep(ps, eta, t_curr, tau):
    """Sakura.get_sakura_tstep (sakura.py:100-117)."""
    dt_a, dt_b = _kern("tstep_kernel", ps, None, {"eta": eta})
    iw2_a = (eta / dt_a) ** 2
    iw2_b = (eta / dt_b) ** 2
    diw2 = (iw2_a - iw2_b)
    w2_sakura = diw2.max()
    dt_sakura = eta / (1 + w2_sakura) ** 0.5
    return block_tstep(abs(dt_sakura), t_curr, tau)


def energies(ps):
    """Kinetic, potential (0.5 sum m phi) energies as body.py:260-321."""
    ke = 0.5 * ps["m"] * (ps["vx"] ** 2 + ps["vy"] ** 2 + ps["vz"] ** 2)
    phi = _kern("phi_kernel", ps)[0]
    pe = ps["m"] * phi
    return float(ke.sum()), 0.5 * float(pe.sum())


def evolve(ps, t_end, eta, method, max_steps=None):
    """Simulation.evolve (simulation.py:191-198) for one method.  Returns the
    list of steps taken; ps is advanced in place."""
    order = {"hermite2": 2, "hermite4": 4, "hermite6": 6, "hermite8": 8}
    t = 0.0
    steps = []
    while abs(t) < t_end:
        tau = base_tstep(t, t_end, eta)
        if "sakura" in method:
            if method == "asakura":
                tau = sakura_tstep(ps, eta, t, tau)
            sakura_step(ps, tau)
        else:
            meth = method[1:] if method.startswith("a") else method
            tau = hermite_step(ps, t, tau, eta, order[meth],
                               method.startswith("a"))
        t += tau
        steps.append(tau)
        if max_steps is not None and len(steps) >= max_steps:
            break
    return steps


# ---------------------------------------------------------------------------
# Individual power-of-two block time steps (not in the reference, whose
# Hermite uses one shared step).  Each particle keeps (t_i, dt_i); at every
# block time t = min(t_i + dt_i) the particles with t_i + dt_i == t are
# active: all particles are predicted to t, the active ones get forces from
# all predicted j, two corrector passes (the second after re-evaluating the
# active particles' forces with their corrected state scattered into the
# predicted set), and a new step from the Tstep kernel quantised with the
# reference's rule (integrator/__init__.py:59-78) at the new time with
# dt_max as the cap.  The forces of the last evaluation become the particle's
# derivatives for its next step.  The device driver follows the same steps.
# ---------------------------------------------------------------------------
DER = {4: ("a", "j"), 6: ("a", "j", "s", "c"), 8: ("a", "j", "s", "c")}


def _pred(order, st, i, dlt):
    """Taylor prediction of r, v, a, j from (t_i) by dlt (fp64)."""
    out = {}
    for c in "xyz":
        r, v, a, j = st["r" + c], st["v" + c], st["a" + c], st["j" + c]
        if order == 4:
            out["r" + c] = r + dlt * (v + dlt * (a + dlt * j / 3) / 2)
            out["v" + c] = v + dlt * (a + dlt * j / 2)
            out["a" + c] = a + dlt * j
            out["j" + c] = j
        else:
            s, cr = st["s" + c], st["c" + c]
            out["r" + c] = r + dlt * (v + dlt * (a + dlt * (j + dlt * (s + dlt * cr / 5) / 4) / 3) / 2)
            out["v" + c] = v + dlt * (a + dlt * (j + dlt * (s + dlt * cr / 4) / 3) / 2)
            out["a" + c] = a + dlt * (j + dlt * (s + dlt * cr / 3) / 2)
            out["j" + c] = j + dlt * (s + dlt * cr / 2)
    return out


def _block_forces(order, I, J):
    """acc/jerk (and snap/crackle) of the i-set I against the j-set J."""
    f = {}
    out = oracle.run("acc_jerk_kernel", I, J)
    for k, v in zip(("ax", "ay", "az", "jx", "jy", "jz"), out):
        f[k] = v
    if order >= 6:
        Ii = dict(I)
        Ii.update(f)
        out = oracle.run("snap_crackle_kernel", Ii, J)
        for k, v in zip(("sx", "sy", "sz", "cx", "cy", "cz"), out):
            f[k] = v
    return f


def block_init(ps, order, eta, dt_max):
    """Forces and steps of all particles at t = 0: acc/jerk first, then (for
    orders 6 and 8) snap/crackle with those a, j on both sides."""
    st = {k: v.copy() for k, v in ps.items() if k in
          ("m", "e2", "rx", "ry", "rz", "vx", "vy", "vz")}
    out = oracle.run("acc_jerk_kernel", st, st)
    for k, v in zip(("ax", "ay", "az", "jx", "jy", "jz"), out):
        st[k] = v
    if order >= 6:
        out = oracle.run("snap_crackle_kernel", st, st)
        for k, v in zip(("sx", "sy", "sz", "cx", "cy", "cz"), out):
            st[k] = v
    dt_a = oracle.run("tstep_kernel", st, st, {"eta": eta})[0]
    st["dt"] = np.array([block_tstep(abs(x), 0.0, dt_max) for x in dt_a])
    st["t"] = np.zeros_like(st["m"])
    return st


def block_step(st, order, eta, dt_max):
    """One block time step; returns (t_new, number of active particles)."""
    t_next = (st["t"] + st["dt"]).min()
    act = np.nonzero(st["t"] + st["dt"] == t_next)[0]
    pr = _pred(order, st, None, t_next - st["t"])
    J = {"m": st["m"], "e2": st["e2"]}
    J.update(pr)
    I0 = {k: st[k][act] for k in st if k not in ("t", "dt")}
    tau = st["dt"][act]
    for it in range(2):
        I = {k: J[k][act] for k in J}
        I["m"] = st["m"][act]
        I["e2"] = st["e2"][act]
        f1 = _block_forces(order, I, J)
        new = {}
        for c in "xyz":
            a0, a1 = I0["a" + c], f1["a" + c]
            j0, j1 = I0["j" + c], f1["j" + c]
            v0, r0 = I0["v" + c], I0["r" + c]
            if order == 4:
                v1 = ((j0 - j1) * tau / 6 + (a0 + a1)) * tau / 2 + v0
                r1 = ((a0 - a1) * tau / 6 + (v0 + v1)) * tau / 2 + r0
            elif order == 6:
                s0, s1 = I0["s" + c], f1["s" + c]
                v1 = (((s0 + s1) * tau / 12 + (j0 - j1)) * tau / 5 + (a0 + a1)) * tau / 2 + v0
                r1 = (((j0 + j1) * tau / 12 + (a0 - a1)) * tau / 5 + (v0 + v1)) * tau / 2 + r0
            else:
                s0, s1 = I0["s" + c], f1["s" + c]
                c0, c1 = I0["c" + c], f1["c" + c]
                v1 = ((((c0 - c1) * tau / 20 + (s0 + s1)) * tau / 3 + 3 * (j0 - j1)) * tau / 14 + (a0 + a1)) * tau / 2 + v0
                r1 = ((((s0 - s1) * tau / 20 + (j0 + j1)) * tau / 3 + 3 * (a0 - a1)) * tau / 14 + (v0 + v1)) * tau / 2 + r0
            new["r" + c] = r1
            new["v" + c] = v1
        for k, v in new.items():
            J[k] = J[k].copy()
            J[k][act] = v
        for k in f1:
            J_k = k
            if k[0] in "aj" and J_k in J:
                J[J_k] = J[J_k].copy()
                J[J_k][act] = f1[k]
    # commit the active particles
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        st[k][act] = J[k][act]
    for k, v in f1.items():
        st[k][act] = v
    I = {k: J[k][act] for k in ("rx", "ry", "rz", "vx", "vy", "vz")}
    I["m"] = st["m"][act]
    I["e2"] = st["e2"][act]
    dt_a = oracle.run("tstep_kernel", I, J, {"eta": eta})[0]
    st["dt"][act] = [block_tstep(abs(x), t_next, dt_max) for x in dt_a]
    st["t"][act] = t_next
    return t_next, len(act)


# ---------------------------------------------------------------------------
# NREG (tupan/integrator/nreg.py): the regularised time transform with
# scalar W, U, S carried between the position and velocity updates.
# ---------------------------------------------------------------------------
def pairwise_sum(a, lo=0, n=None):
    """numpy's add.reduce order for a contiguous float64 array: below 8
    elements a sequential sum from 0.0; up to 128 elements eight running
    sums over strided elements, combined as ((r0+r1)+(r2+r3))+((r4+r5)+
    (r6+r7)), then the tail; above that the two halves (the first rounded
    down to a multiple of 8) summed recursively and added."""
    if n is None:
        n = len(a)
    if n < 8:
        res = 0.0
        for i in range(n):
            res += a[lo + i]
        return res
    if n <= 128:
        r = [a[lo + j] for j in range(8)]
        i = 8
        while i < n - (n % 8):
            for j in range(8):
                r[j] += a[lo + i + j]
            i += 8
        res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
        while i < n:
            res += a[lo + i]
            i += 1
        return res
    n2 = n // 2
    n2 -= n2 % 8
    return pairwise_sum(a, lo, n2) + pairwise_sum(a, lo + n2, n - n2)


class NregState(object):
    """ParticleSystem class attributes the reference keeps for NREG."""

    def __init__(self, ps):
        self.t = 0.0
        mtot = float(ps["m"].sum())
        k, p = energies(ps)
        self.E0 = k + p
        self.W = -p
        self.U = -p
        self.S = -p
        self.mtot = mtot


def nreg_x(ps, st, dt):
    """nreg.py:22-34"""
    out = _kern("nreg_Xkernel", ps, None, {"dt": dt})
    for k, v in zip(("mrx", "mry", "mrz", "ax", "ay", "az", "u"), out):
        ps[k] = v
    mtot = float(ps["m"].sum())
    for c in "xyz":
        ps["r" + c] = ps["mr" + c] / mtot
    st.U = 0.5 * ps["u"].sum()
    st.t += dt


def nreg_v(ps, st, dt):
    """nreg.py:46-57"""
    out = _kern("nreg_Vkernel", ps, None, {"dt": dt})
    for k, v in zip(("mvx", "mvy", "mvz", "mk"), out):
        ps[k] = v
    mtot = float(ps["m"].sum())
    for c in "xyz":
        ps["v" + c] = ps["mv" + c] / mtot
    K = 0.25 * ps["mk"].sum() / mtot
    st.W = (K - st.E0)


def anreg_step(ps, st, h):
    """nreg.py:77-86"""
    nreg_x(ps, st, 0.5 * (h / st.W))
    nreg_v(ps, st, (h / st.U))
    nreg_x(ps, st, 0.5 * (h / st.W))


def nreg_step(ps, st, h):
    """nreg.py:89-98"""
    anreg_step(ps, st, 0.5 * (h * st.S))
    st.S = 1 / (2 / st.W - 1 / st.S)
    anreg_step(ps, st, 0.5 * (h * st.S))


def nreg_evolve(ps, t_end, eta, method, max_steps=None):
    """NREG.initialize + the evolve loop over NREG.do_step (nreg.py:111-
    170).  Returns (state scalars, list of t after each step); ps (a dict
    with ax, ay, az zero-initialised if absent) is advanced in place."""
    for k in ("ax", "ay", "az"):
        ps.setdefault(k, np.zeros(len(ps["m"])))
    st = NregState(ps)
    times = []
    while abs(st.t) < t_end:
        tau = base_tstep(st.t, t_end, eta)
        if "anreg" in method:
            anreg_step(ps, st, tau / 2)
        else:
            nreg_step(ps, st, tau)
        times.append(st.t)
        if max_steps is not None and len(times) >= max_steps:
            break
    return st, times
