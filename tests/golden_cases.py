"""Read the golden fixtures written by tests/golden/make_golden.py."""

import glob
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CUT = {"all": slice(None), "j37": slice(0, 37), "i37": slice(0, 37),
       "i5": slice(0, 5), "i1": slice(0, 1)}

SCALARS = {
    "tstep_kernel": lambda a: {"eta": a[0]},
    "nreg_Xkernel": lambda a: {"dt": a[0]},
    "nreg_Vkernel": lambda a: {"dt": a[0]},
    "sakura_kernel": lambda a: {"dt": a[0], "flag": a[1]},
}
C = 128.0
PN = dict(order=7, **{"inv%d" % k: (1.0 / C) ** k for k in range(1, 8)})


def files():
    return sorted(glob.glob(os.path.join(HERE, "golden_*_float*.npz")))


def load(path):
    z = np.load(path)
    prec = str(z["__prec__"])
    data = {k[3:]: z[k] for k in z.files if k.startswith("in/")}
    cases = {}
    for k in z.files:
        if not k.startswith("out/"):
            continue
        tag, idx = k[4:].rsplit("/", 1)
        cases.setdefault(tag, {})[int(idx)] = z[k]
    out = []
    for tag, res in sorted(cases.items()):
        name, ir, jr, args = tag.split("|")
        args = tuple(eval(a) for a in args.split(",")) if args else ()
        if name == "pnacc_kernel":
            scalars = dict(PN)
        else:
            scalars = SCALARS.get(name, lambda a: {})(args)
        ips = {a: v[CUT[ir]] for a, v in data.items()}
        jps = {a: v[CUT[jr]] for a, v in data.items()}
        expect = tuple(res[i] for i in range(len(res)))
        out.append((tag, name, ips, jps, scalars, expect))
    kepler = []
    for k in z.files:
        if k.startswith("kepler/"):
            dt = eval(k[len("kepler/"):])
            pairs = z["kepler_pairs/%r" % dt]
            kepler.append((dt, pairs, z[k]))
    return prec, data, out, kepler
