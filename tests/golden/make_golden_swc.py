#!/usr/bin/env python3
"""SWC fixtures and what the REFERENCE builds from them.

1. Writes seeded synthetic SWC files under ``tests/golden/swc/`` (random
   dendritic trees grown here; no third-party morphology): soma with
   several primary dendrites, forks of up to four children, axon / apical
   types, zero-length segments (exactly on, and within 0.01 um of, their
   parent), comment and blank lines, tabs, mixed number formats, CRLF line
   ends, bad lines at the end of a file, and three files that fail
   validation (two roots, a parent after its child, a radius below
   0.04 um).
2. Loads each with the reference ``moose.loadModel`` (``ReadSwc`` +
   ``ReadSwc::build``, RM 1, RA 1, CM 0.01) and records, in creation order,
   every compartment's name, parent, children (message order), Ra, Rm, Cm,
   diameter, length, Em, initVm and coordinates, plus ReadSwc's own summary
   line (segments, bad lines, validated, branches).
3. For each valid file: soma inject 0.2 nA, an HSolve with target = soma,
   2,000 steps of 25 us; records the final Vm of every compartment and the
   soma / last compartment traces (every 10th step).

Output: ``tests/golden/swc_golden.npz``.  Prerequisite: the reference build
(``python oracle/build_ref.py``); run from anywhere.
"""
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
SWC_DIR = os.path.join(HERE, "swc")
DT, NSTEPS, INJECT, STRIDE = 25e-6, 2000, 0.2e-9, 10


def _fmt(rng, v):
    k = int(rng.integers(4))
    return ("%.4f" % v, "%g" % v, "%.6e" % v, "%.2f" % v)[k]


def synth_swc(seed, n, n_primary=3, max_kids=2, branch_p=0.15, zero_p=0.0, types=(3,), soma_r=6.0,
              crlf=False, noise=False, tail_bad=False):
    """A random tree of n segments grown from a soma at the origin."""
    rng = np.random.default_rng(seed)
    segs = [[1, 1, 0.0, 0.0, 0.0, soma_r, -1]]
    tips = []
    for k in range(n_primary):
        th = 2 * np.pi * k / n_primary + rng.uniform(-0.2, 0.2)
        d = np.array([np.cos(th), np.sin(th), rng.uniform(-0.3, 0.3)])
        d /= np.linalg.norm(d)
        t = types[k % len(types)]
        p = d * (soma_r + rng.uniform(1.0, 4.0))
        segs.append([len(segs) + 1, t, p[0], p[1], p[2], rng.uniform(0.8, 1.6), 1])
        tips.append((len(segs), d, t))
    while len(segs) < n:
        idx, d, t = tips.pop(int(rng.integers(len(tips))))
        par = segs[idx - 1]
        if rng.random() < zero_p:
            # a zero-length segment: on its parent, or within 0.01 um of it
            off = 0.0 if rng.random() < 0.5 else 0.004
            segs.append([len(segs) + 1, t, par[2] + off, par[3], par[4], par[5], idx])
            tips.append((len(segs), d, t))
            continue
        k = 1
        if rng.random() < branch_p:
            k = int(rng.integers(2, max_kids + 1))
        for _ in range(k):
            if len(segs) >= n:
                break
            dd = d + rng.normal(0, 0.35, 3)
            dd /= np.linalg.norm(dd)
            step = rng.uniform(2.0, 12.0)
            r = max(0.05, par[5] * rng.uniform(0.85, 1.0))
            segs.append([len(segs) + 1, t, par[2] + step * dd[0], par[3] + step * dd[1], par[4] + step * dd[2],
                         r, idx])
            tips.append((len(segs), dd, t))
    lines = ["# synthetic morphology, seed %d" % seed, "# n T x y z R P"]
    for i, s in enumerate(segs):
        fields = ["%d" % s[0], "%d" % s[1]] + [_fmt(rng, v) for v in s[2:6]] + ["%d" % s[6]]
        sep = "\t" if noise and rng.random() < 0.2 else " "
        line = sep.join(fields)
        if noise and rng.random() < 0.1:
            line = "  " + line + "   "
        lines.append(line)
        if noise and rng.random() < 0.03:
            lines.append("")
        if noise and rng.random() < 0.03:
            lines.append("   # a comment inside")
    if tail_bad:
        lines += ["%d 3 1.0 2.0 3.0 1.0" % (len(segs) + 1),            # six fields
                  "%d 7 1.0 2.0 3.0 1.0 1" % (len(segs) + 1),          # custom type
                  "%d 0 1.0 2.0 3.0 1.0 1" % (len(segs) + 1)]          # undefined type
    eol = "\r\n" if crlf else "\n"
    return eol.join(lines) + eol


def fixtures():
    return {
        "tree_basic": synth_swc(11, 120),
        "tree_forks4": synth_swc(12, 400, n_primary=4, max_kids=4, branch_p=0.25, types=(3, 4, 2)),
        "tree_zero_length": synth_swc(13, 250, n_primary=3, max_kids=3, branch_p=0.2, zero_p=0.05,
                                      types=(4, 3)),
        "tree_noisy_crlf": synth_swc(14, 200, n_primary=5, branch_p=0.2, crlf=True, noise=True, tail_bad=True,
                                     types=(2, 3, 3, 4, 3)),
        "tree_axon_long": synth_swc(15, 600, n_primary=2, branch_p=0.05, types=(2, 3)),
        "invalid_two_roots": synth_swc(16, 30) + "31 1 50 50 50 5 -1\n",
        "invalid_orphan": synth_swc(17, 30) + "31 3 1 1 1 1 40\n",
        "invalid_radius": synth_swc(18, 30) + "31 3 1 1 1 0.01 30\n",
    }


def _capture(fn):
    """Run fn() with the C-level stdout sent to a file; return (result, text)."""
    sys.stdout.flush()
    fd = os.dup(1)
    with tempfile.TemporaryFile(mode="w+") as tmp:
        os.dup2(tmp.fileno(), 1)
        try:
            r = fn()
        finally:
            sys.stdout.flush()
            os.dup2(fd, 1)
            os.close(fd)
        tmp.seek(0)
        return r, tmp.read()


def reference_load(path, where):
    import moose
    model, text = _capture(lambda: moose.loadModel(path, where))
    m = re.search(r"NumSegs = (\d+), bad = (\d+), Validated = (\d+), numBranches = (\d+)", text)
    summary = np.array([int(g) for g in m.groups()])
    cs = moose.wildcardFind(where + "/#[ISA=CompartmentBase]")
    cs.sort(key=lambda c: int(re.search(r"id=(\d+)", str(c.id)).group(1)))     # creation order
    return model, cs, summary


def make():
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    import moose
    os.makedirs(SWC_DIR, exist_ok=True)
    out = {}
    for k, (name, text) in enumerate(sorted(fixtures().items())):
        path = os.path.join(SWC_DIR, name + ".swc")
        with open(path, "w", newline="") as f:
            f.write(text)
        where = "/swc%d" % k
        model, cs, summary = reference_load(path, where)
        names = [c.name for c in cs]
        idx = {c: i for i, c in enumerate(names)}
        out[name + "/summary"] = summary
        out[name + "/names"] = np.array(names)
        out[name + "/parent"] = np.array([idx[c.neighbors["raxial"][0].name] if len(c.neighbors["raxial"]) else -1
                                          for c in cs], np.int32)
        out[name + "/children"] = np.array([",".join(x.name for x in c.neighbors["axial"]) for c in cs])
        for f in ("Ra", "Rm", "Cm", "diameter", "length", "Em", "initVm", "x0", "y0", "z0", "x", "y", "z"):
            out[name + "/" + f] = np.array([getattr(c, f) for c in cs], np.float64)
        if not cs:
            moose.delete(where)
            continue
        soma = moose.element(where + "/soma")
        soma.inject = INJECT
        for t in range(8):
            moose.setClock(t, DT)
        moose.setClock(8, DT * STRIDE)
        rec = [cs[0], cs[-1]]
        tabs = []
        for i, c in enumerate(rec):
            t = moose.Table("%s/vm%d" % (where, i))
            moose.connect(t, "requestOut", c, "getVm")
            tabs.append(t)
        h = moose.HSolve(where + "/hsolve")
        h.dt = DT
        h.target = soma.path
        moose.reinit()
        moose.start(NSTEPS * DT)
        out[name + "/trace"] = np.array([t.vector for t in tabs])
        out[name + "/final_vm"] = np.array([c.Vm for c in cs])
        moose.delete(where)
    np.savez_compressed(os.path.join(HERE, "swc_golden.npz"), dt=DT, nsteps=NSTEPS, inject=INJECT, stride=STRIDE,
                        **out)
    print("wrote", os.path.join(HERE, "swc_golden.npz"))


if __name__ == "__main__":
    make()
