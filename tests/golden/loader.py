"""Rebuild the CellModel stored in a golden .npz (keys written by
make_golden_active.save_model) so that any machine steps bit-identical input."""
import numpy as np


def load_model(z, prefix="model_"):
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__)))), "moose-core_gb300"))
    from moose_gb300.abi import CellModel, _ARRAYS
    # fixtures written before an array existed describe cells without it
    kw = {k: z[prefix + k] for k in _ARRAYS if prefix + k in z.files}
    gates = []
    for i in range(int(z[prefix + "ngates"])):
        AB = z[prefix + "gate%d" % i]
        mn, mx = z[prefix + "gate%d_range" % i]
        gates.append((float(mn), float(mx), AB[0], AB[1]))
    gates2d = []
    for i in range(int(z[prefix + "ngates2d"])):
        AB = z[prefix + "gate2d%d" % i]
        r = z[prefix + "gate2d%d_range" % i]
        gates2d.append((float(r[0]), float(r[1]), float(r[2]), float(r[3]), AB[0], AB[1]))
    meta = {k[5:]: z[k] for k in z.files if k.startswith("meta_")}
    return CellModel(seed=int(z[prefix + "seed"]), gates=gates, gates2d=gates2d, meta=meta, **kw)


def replay_messages(z, solver, per_step):
    """Drive `solver` (oracle or GPU drop-in) with the values the reference's
    StimulusTables sent at each step (inject, external conc, Ca current) and
    sample Vm/Ca like the reference's Tables."""
    rec, recp = z["rec"], z["rec_pool"]
    stride, n = int(z["stride"]), int(z["nsteps"])
    vm, ca = [solver.vm()[rec]], [solver.ca()[recp]]
    for k in range(n):
        solver.add_inject(0, z["sent_inject"][k])
        for c in z["ext"]:
            solver.add_conc(int(c), z["sent_conc"][k])
        solver.add_ica(0, z["sent_ica"][k])
        per_step(solver)
        if (k + 1) % stride == 0:
            vm.append(solver.vm()[rec])
            ca.append(solver.ca()[recp])
    return np.array(vm).T, np.array(ca).T



def push_pre_reinit(z, solver):
    """The events active_events.npz pushed before reinit (synapse 1 of each
    SynChan, delay added as Synapse::addSpike adds it); reinit drops them."""
    k = z["pre_syn"]
    solver.push_events(k, z["pre_time"] + z["syn_delay"][k, 1], z["syn_weight"][k, 1])


def replay_events(z, solver, advance):
    """Drive `solver` (oracle or GPU drop-in, after reinit) through
    active_events.npz: `advance(solver, n)` steps it, and once `push_step`
    steps have run the events of that chunk are pushed with time = spike
    time + synapse delay and the synapse's weight.  Returns the Vm samples
    of the reference's Tables (every `stride` steps, sample 0 at reinit)."""
    w, dl = z["syn_weight"], z["syn_delay"]
    ps, pk, pj, pt = z["push_step"], z["push_syn"], z["push_synapse"], z["push_time"]
    rec, stride, n = z["rec"], int(z["stride"]), int(z["nsteps"])
    vm = [solver.vm()[rec]]
    for cur in range(0, n, stride):
        sel = ps == cur
        if sel.any():
            solver.push_events(pk[sel], pt[sel] + dl[pk[sel], pj[sel]], w[pk[sel], pj[sel]])
        advance(solver, stride)
        vm.append(solver.vm()[rec])
    return np.array(vm).T


def model_from_desc(d, seed):
    """A CellModel holding a copy of every array of the HsCellDesc `d` (a
    ctypes structure, e.g. one the MOOSE-side binding filled), seeded at
    `seed`."""
    import ctypes as C
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__)))), "moose-core_gb300"))
    from moose_gb300.abi import CellModel, HS_DIF_NPAR, _ARRAYS, _COUNTS
    count_of = {first: getattr(d, cnt) for cnt, first in _COUNTS.items()}
    kw = {}
    for name, dt in _ARRAYS.items():
        if name == "difpar":
            n = HS_DIF_NPAR * d.n_dif
        else:
            prefix = name.split("_")[0] + "_"
            first = next((f for f in _COUNTS.values() if f.startswith(prefix)), "parent")
            n = count_of[first] if name not in ("Ra", "Rm", "Cm", "Em", "initVm", "Vm", "inject") else d.n_compt
        p = getattr(d, name)
        kw[name] = np.ctypeslib.as_array(p, shape=(n,)).astype(dt).copy() if n and p else np.zeros(0, dt)
    gates = []
    for i in range(d.n_gate):
        g = d.gate[i]
        A = np.ctypeslib.as_array(g.A, shape=(g.divs + 1,)).copy()
        B = np.ctypeslib.as_array(g.B, shape=(g.divs + 1,)).copy()
        gates.append((g.min, g.max, A, B))
    gates2d = []
    for i in range(d.n_gate2d):
        g = d.gate2d[i]
        shape = (g.xdivs + 1, g.ydivs + 1)
        A = np.ctypeslib.as_array(g.A, shape=(shape[0] * shape[1],)).reshape(shape).copy()
        B = np.ctypeslib.as_array(g.B, shape=(shape[0] * shape[1],)).reshape(shape).copy()
        gates2d.append((g.xmin, g.xmax, g.ymin, g.ymax, A, B))
    return CellModel(seed=int(seed), gates=gates, gates2d=gates2d, **kw)
