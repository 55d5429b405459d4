"""The plain form's wavefront schedule of lexicographic line sweeps
(trans_bl_gb300/csrc/tb_plain.cu, k_wsor) restated in Python and checked
against the reference's sequential order (sor, poisson_par.f:167-226) on a
model problem: each line update is a nonlinear function of the lines its
stencil reads, so any read of a value from the wrong sweep changes the
result.  Also checks that the 32-line shared-memory ring holds every line a
step touches."""
import numpy as np
import pytest

LAG, RING, MAX_STREAM = 5, 32, 5


def update(kind, F, i, m):
    """New value of line i from the lines its stencil reads (model of one line solve)."""
    if kind == "c":
        nb = (F[i - 2], F[i - 1], F[i + 1], F[i + 2])
    elif kind == "b1":
        nb = (F[0], F[2], F[3], F[4], F[5])
    else:
        nb = (F[m + 1], F[m - 1], F[m - 2], F[m - 3], F[m - 4])
    w = np.array([0.31, 0.17, 0.23, 0.11, 0.07][:len(nb)])
    return np.sin(F[i] + sum(a * b for a, b in zip(w, nb))) + 0.01 * i


def sequential(F, ns):
    F = F.copy()
    nxl = F.shape[0]
    m = nxl - 2
    for _ in range(ns):
        F[1] = update("b1", F, 1, m)
        F[m] = update("b2", F, m, m)
        for i in range(2, m):
            F[i] = update("c", F, i, m)
    return F


def wavefront(F, ns, whole):
    """k_wsor's schedule: sweep s runs border1 at step LAG*s, the centre line
    u+1 at step u+LAG*s, border2 at step m-6+LAG*s; tasks of one step are
    computed from the state before the step (they must be independent)."""
    G = F.copy()
    nxl = F.shape[0]
    m = nxl - 2
    T = m - 1 + LAG * (ns - 1)
    ring = {}
    loaded, stored = -1, 0
    for t in range(T):
        if not whole:
            hi = min(nxl - 1, t + 7)
            lo = max(0, t - 1 - LAG * (ns - 1))
            for line in range(stored, lo):
                G[line] = ring.pop(line)
            for line in range(loaded + 1, hi + 1):
                assert all((q % RING) != (line % RING) for q in ring), "ring slot reused while live"
                ring[line] = G[line].copy()
            stored, loaded = lo, hi
            view = ring
        else:
            view = {q: G[q] for q in range(nxl)}
        tasks = []
        for s in range(ns):
            u = t - LAG * s
            if u == 0:
                tasks.append(("b1", 1, (0, 2, 3, 4, 5)))
            if 1 <= u <= m - 2:
                i = u + 1
                tasks.append(("c", i, (i - 2, i - 1, i + 1, i + 2)))
            if u == m - 6:
                tasks.append(("b2", m, (m + 1, m - 1, m - 2, m - 3, m - 4)))
        writes = [i for _, i, _ in tasks]
        assert len(set(writes)) == len(writes)
        for _, i, reads in tasks:
            for q in reads + (i,):
                assert q in view, "line %d not resident at step %d" % (q, t)
                assert q == i or q not in writes, "step %d reads line %d another task writes" % (t, q)
        snap = {q: view[q].copy() for q in view}
        new = {i: update(kind, snap, i, m) for kind, i, _ in tasks}
        for i, v in new.items():
            view[i][...] = v
    if not whole:
        for line in range(stored, loaded + 1):
            G[line] = ring.pop(line)
    return G


@pytest.mark.parametrize("nxl", [9, 10, 13, 33, 65, 97])
@pytest.mark.parametrize("ns", [1, 2, 3, 5, 60])
def test_wavefront_equals_sequential(nxl, ns):
    rng = np.random.default_rng(nxl * 100 + ns)
    F = rng.standard_normal((nxl, 7))
    ref = sequential(F, ns)
    if ns <= MAX_STREAM:
        np.testing.assert_array_equal(wavefront(F, ns, whole=False), ref)
    np.testing.assert_array_equal(wavefront(F, ns, whole=True), ref)
