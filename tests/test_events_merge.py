"""The host merge behind hs_push_events (hsg::mergeEventQueue,
moose-core_gb300/csrc/hs_events.h), compiled here with g++ through
tests/cpp/events_merge_shim.cpp: SimpleSynHandler::addSpike queues
(synapse/SimpleSynHandler.cpp:86-90) rebuilt from the device cursors.

* exact agreement with a Python model of the merge: per SynChan the
  undelivered events and the pushed ones in time order, queued events first
  on equal times, pushed ones in push order; delivered events dropped;
  cursors clamped into each SynChan's range;
* a run of rounds (push, deliver up to the step's clock time, merge) gives
  each step the activation a min-heap of (time, push sequence) gives, the
  sums taken in the same order -- SimpleSynHandler::vProcess.
"""
import ctypes as C
import heapq
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "cpp", "_build")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "cpp", "events_merge_shim.cpp")
    hdr = os.path.join(REPO, "moose-core_gb300", "csrc", "hs_events.h")
    so = os.path.join(OUT, "libevents_merge_shim.so")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-fPIC", "-shared", "-o", so, src,
                        "-I", os.path.join(REPO, "moose-core_gb300", "csrc")], check=True, capture_output=True,
                       text=True)
    L = C.CDLL(so)
    pu, pd = C.POINTER(C.c_uint32), C.POINTER(C.c_double)
    L.merge_events.argtypes = [C.c_uint32, pu, pd, pd, pu, C.c_uint32, pu, pd, pd, C.c_uint32, pu, pd, pd, pu]
    L.merge_events.restype = C.c_int
    return L


def _u(a):
    return np.ascontiguousarray(a, np.uint32)


def _d(a):
    return np.ascontiguousarray(a, np.float64)


def merge(L, S, ptr, t, w, cur, ps, pt, pw):
    ptr, cur, ps = _u(ptr), _u(cur), _u(ps)
    t, w, pt, pw = _d(t), _d(w), _d(pt), _d(pw)
    cap = int(ptr[S]) + len(ps) + 1
    op, ot, ow, n = np.zeros(2 * S + 1, np.uint32), np.zeros(cap), np.zeros(cap), C.c_uint32()
    P = lambda a, ty: a.ctypes.data_as(C.POINTER(ty))
    rc = L.merge_events(S, P(ptr, C.c_uint32), P(t, C.c_double), P(w, C.c_double), P(cur, C.c_uint32),
                        len(ps), P(ps, C.c_uint32), P(pt, C.c_double), P(pw, C.c_double), cap,
                        P(op, C.c_uint32), P(ot, C.c_double), P(ow, C.c_double), C.byref(n))
    assert rc == 0
    return op, ot[:n.value], ow[:n.value]


def model(S, ptr, t, w, cur, ps, pt, pw):
    out_ptr, out_t, out_w = [], [], []
    for k in range(S):
        c = min(max(int(cur[k]), int(ptr[k])), int(ptr[k + 1]))
        q = [(t[e], 0, e, w[e]) for e in range(c, int(ptr[k + 1]))]
        q += [(pt[i], 1, i, pw[i]) for i in range(len(ps)) if ps[i] == k]
        q.sort(key=lambda x: (x[0], x[1], x[2]))
        out_ptr.append(len(out_t))
        out_t += [x[0] for x in q]
        out_w += [x[3] for x in q]
    out_ptr.append(len(out_t))
    return np.array(out_ptr + out_ptr[:S], np.uint32), np.array(out_t), np.array(out_w)


def random_queue(rng, S, ties):
    counts = rng.integers(0, 6, S)
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    t = np.concatenate([np.sort(rng.choice([0.1, 0.2, 0.3], c) if ties else rng.uniform(0, 1, c))
                        for c in counts]) if counts.sum() else np.zeros(0)
    w = rng.uniform(0.1, 1.0, int(ptr[-1]))
    cur = np.array([rng.integers(ptr[k], ptr[k + 1] + 1) for k in range(S)], np.uint32)
    return ptr, t, w, cur


@pytest.mark.parametrize("seed", range(8))
def test_merge_matches_model(lib, seed):
    rng = np.random.default_rng(seed)
    S = int(rng.integers(1, 12))
    ties = seed % 2 == 0
    ptr, t, w, cur = random_queue(rng, S, ties)
    n = int(rng.integers(0, 30))
    ps = rng.integers(0, S, n)
    pt = rng.choice([0.1, 0.2, 0.3, 0.25], n) if ties else rng.uniform(-0.5, 1.5, n)
    pw = rng.uniform(0.1, 1.0, n)
    got = merge(lib, S, ptr, t, w, cur, ps, pt, pw)
    want = model(S, ptr, t, w, cur, ps, pt, pw)
    for g, m in zip(got, want):
        assert np.array_equal(g, m)


def test_cursors_are_clamped(lib):
    ptr = np.array([0, 2, 4], np.uint32)
    t, w = np.array([0.1, 0.2, 0.3, 0.4]), np.array([1.0, 2.0, 3.0, 4.0])
    got = merge(lib, 2, ptr, t, w, np.array([7, 0], np.uint32), [1], [0.35], [9.0])
    assert np.array_equal(got[0], [0, 0, 3, 0, 0])
    assert np.array_equal(got[1], [0.3, 0.35, 0.4])
    assert np.array_equal(got[2], [3.0, 9.0, 4.0])


def test_rounds_deliver_like_a_heap(lib):
    """Push between steps, deliver every event with time <= the step's
    clock time (dt * step) as weight/dt, merge at each push: per-step
    activations equal those of a (time, sequence) min-heap per SynChan."""
    rng = np.random.default_rng(11)
    S, dt, steps = 5, 0.25, 400
    ptr = np.zeros(S + 1, np.uint32)
    t, w = np.zeros(0), np.zeros(0)
    cur = np.zeros(S, np.uint32)
    heaps = [[] for _ in range(S)]
    seq = 0
    for step in range(steps):
        if step % 7 == 0:
            n = int(rng.integers(0, 12))
            ps = rng.integers(0, S, n)
            pt = dt * step + rng.uniform(-2.0, 6.0, n)      # late events too
            pw = rng.uniform(0.1, 1.0, n)
            for k, a, b in zip(ps, pt, pw):
                heapq.heappush(heaps[k], (a, seq, b))
                seq += 1
            op, t, w = merge(lib, S, ptr, t, w, cur, ps, pt, pw)
            ptr, cur = op[:S + 1].copy(), op[S + 1:].copy()
        now = dt * (step + 1)
        for k in range(S):
            act = 0.0
            while cur[k] < ptr[k + 1] and t[cur[k]] <= now:
                act += w[cur[k]] / dt
                cur[k] += 1
            ref = 0.0
            while heaps[k] and heaps[k][0][0] <= now:
                ref += heapq.heappop(heaps[k])[2] / dt
            assert act == ref
