"""CPU emulation of the dataflow schedule of the cluster LDL^T
(mcvslam_gb300/csrc/mcba_chol_dev.cuh): the per-CTA task lists of worker_tasks(),
the version-flag conditions of load_task() and of the chain CTA, and the
tile-major workspace.  The CTAs step in random interleavings, each task runs
only when its flags say its inputs are ready, and the test checks that

* every panel, trailing update and inverse appears exactly once;
* no interleaving deadlocks (a CTA whose next task is not ready waits, as
  the kernel's in-order waits do);
* no task reads a tile that no producer has written (NaN-filled workspace);
* the backward solve's result equals numpy's solve.

The lookahead worker's two tiles of block row k+2, which the kernel pushes
into the chain CTA's shared memory, are modelled as flagged workspace tiles
that the chain CTA reads; the ordering is the same (the push happens after
the chain CTA's panel flag of step k)."""
import numpy as np
import pytest

B = 16


def task_lists(nblk, C):
    """Per-worker task lists: lists[0..C-3] the general workers (dealt round
    robin over one global order), lists[C-2] the lookahead worker."""
    W = C - 2
    lists = [[] for _ in range(W + 1)]
    m = [0]

    def seg(cnt, f):
        for idx in range(max(cnt, 0)):
            lists[(m[0] + idx) % W].append(f(idx))
        m[0] += max(cnt, 0)

    for k in range(nblk):
        if k + 2 <= nblk:
            r = k + 2
            tl = [("panel", r, k), ("upd", r, k + 1, k)]
            if r < nblk:
                tl.append(("upd", r, r, k))
            tl.append(("inv", k))
            lists[W].extend(tl)
        if k + 1 < nblk:
            seg(nblk - k - 2, lambda idx: ("panel", k + 3 + idx, k))
            seg(nblk - k - 2, lambda idx: ("upd", k + 3 + idx, k + 1, k))
        if k + 2 < nblk:
            seg(nblk - k - 2, lambda idx: ("upd", k + 3 + idx, k + 2, k))
        if k >= 1 and k + 3 < nblk:
            cnt = sum(nblk - j + 1 for j in range(k + 3, nblk))

            def deferred(idx, k=k):
                j = k + 3
                while idx >= nblk - j + 1:
                    idx -= nblk - j + 1
                    j += 1
                return ("upd", j + idx, j, k - 1)

            seg(cnt, deferred)
        if k + 3 < nblk:
            seg(nblk - k - 2, lambda idx: ("upd", k + 3 + idx, k + 3, k))
    return lists


def expected_tasks(nblk):
    exp = set()
    for j in range(nblk):
        for s in range(j):
            for i in range(j, nblk + 1):
                if not (i == j == s + 1):  # the chain CTA updates diagonal tile s+1 itself
                    exp.add(("upd", i, j, s))
    for k in range(nblk):
        for i in range(k + 2, nblk + 1):  # panel (k+1, k) is the chain CTA's
            exp.add(("panel", i, k))
    for J in range(nblk - 1):  # the last inverse is the chain CTA's
        exp.add(("inv", J))
    return exp


def ldlt_tile(T):
    """LDL^T of a symmetric tile given by its lower part: strict lower <- L,
    diagonal <- d, and 1/d."""
    M = np.tril(T) + np.tril(T, -1).T
    L = np.eye(B)
    d = np.zeros(B)
    for j in range(B):
        d[j] = M[j, j] - (L[j, :j] ** 2 * d[:j]).sum()
        for i in range(j + 1, B):
            L[i, j] = (M[i, j] - (L[i, :j] * L[j, :j] * d[:j]).sum()) / d[j]
    return np.tril(L, -1) + np.diag(d), 1.0 / d


def emulate(n, C, seed):
    rng = np.random.default_rng(seed)
    ld = 32 * ((n + 31) // 32)
    nblk = (n + B - 1) // B
    A = rng.standard_normal((n, n))
    A = A @ A.T + n * np.eye(n)
    b = rng.standard_normal(n)
    S = np.zeros((ld + 32, ld))
    S[:n, :n] = A
    for i in range(n, ld):
        S[i, i] = 1.0
    S[ld, :n] = b
    ws = np.full((ld + 32, ld), np.nan)  # rows ld+1, ld+2: 1/d and y
    fl = {}
    Ms = {}
    Ps = {}

    def flag(key):
        return fl.get(key, 0)

    def tile(i, j):  # working tile (i, j); block row nblk is the right-hand side
        return (slice(B * i, B * i + B), slice(B * j, B * j + B)) if i < nblk else (ld, slice(B * j, B * j + B))

    def upper(i, j):  # L_ij sits at (j, i)
        return (slice(B * j, B * j + B), slice(B * i, B * i + B))

    def read(i, j, v):
        t = (S if v == 0 else ws)[tile(i, j)].copy()
        assert not np.isnan(t).any(), ("read before write", i, j, v)
        return t

    lists = task_lists(nblk, C)
    allt = [t for lst in lists for t in lst]
    assert len(allt) == len(set(allt))
    assert set(allt) == expected_tasks(nblk)

    def ready(t):  # load_task's flag conditions
        if t[0] == "inv":  # diagonal tile J factored, the chain's panel (J+1, J)
            J = t[1]
            return flag((J, J)) >= J + 1 and (J + 1 == nblk or flag((J + 1, J)) >= J + 1)
        if t[0] == "panel":
            _, i, k = t
            return (k == 0 or flag((i, k)) >= k) and flag((k, k)) >= k + 1
        _, i, j, s = t
        return (s == 0 or flag((i, j)) >= s) and flag((i, s)) >= s + 1 and flag((j, s)) >= s + 1

    def execute(t):
        if t[0] == "inv":
            J = t[1]
            Lu = np.tril(ws[tile(J, J)], -1) + np.eye(B)
            Ms[J] = np.linalg.inv(Lu).T
            if J + 1 < nblk:  # P_J = M_J L_{J+1,J}^T
                Lt = ws[upper(J + 1, J)].copy()
                assert not np.isnan(Lt).any(), ("inverse reads an unwritten panel", J)
                Ps[J] = Ms[J] @ Lt.T
            fl[("inv", J)] = 1
            return
        if t[0] == "panel":
            _, i, k = t
            Lu = np.tril(ws[tile(k, k)], -1) + np.eye(B)
            rd = ws[ld + 1, B * k:B * k + B].copy()
            a = read(i, k, k)
            if i < nblk:
                Wt = np.linalg.solve(Lu, a.T).T
                ws[tile(i, k)] = Wt
                ws[upper(i, k)] = Wt * rd[None, :]
            else:
                Wt = np.linalg.solve(Lu, a)
                ws[ld, B * k:B * k + B] = Wt
                ws[ld + 2, B * k:B * k + B] = Wt * rd
            fl[(i, k)] = k + 1
            return
        _, i, j, s = t
        a = read(i, j, s)
        Wt = ws[tile(i, s)].copy()
        Lt = ws[upper(j, s)].copy()
        assert not np.isnan(Wt).any() and not np.isnan(Lt).any()
        if i < nblk:
            r = a - Wt @ Lt.T
            if i == j:
                r = np.where(np.tril(np.ones((B, B))) > 0, r, a)
        else:
            r = a - Lt @ Wt
        ws[tile(i, j)] = r
        fl[(i, j)] = s + 1

    st = {"k": 0, "phase": "factor", "T": S[0:B, 0:B].copy()}

    def chain_step():
        k = st["k"]
        more = k + 1 < nblk
        if st["phase"] == "factor":
            # the tiles (k+1, k) and (k+1, k+1) at version k (the lookahead push)
            if more and k > 0 and not (flag((k + 1, k)) >= k and flag((k + 1, k + 1)) >= k):
                return False
            if not more and k > 0 and flag((nblk, k)) < k:
                return False
            Tf, rd = ldlt_tile(st["T"])
            ws[tile(k, k)] = Tf
            ws[ld + 1, B * k:B * k + B] = rd
            fl[(k, k)] = k + 1
            Lu = np.tril(Tf, -1) + np.eye(B)
            if not more:
                st["ylast"] = np.linalg.solve(Lu, read(nblk, k, k)) * rd
                Ms[k] = np.linalg.inv(Lu).T
                st["phase"] = "backward"
                return True
            Wt = np.linalg.solve(Lu, read(k + 1, k, k).T).T
            Lt = Wt * rd[None, :]
            Q = read(k + 1, k + 1, k) - np.tril(Wt @ Lt.T)
            ws[tile(k + 1, k)] = Wt
            ws[upper(k + 1, k)] = Lt
            fl[(k + 1, k)] = k + 1
            st["T"] = Q
            st["k"] = k + 1
            return True
        if st["phase"] == "backward":
            if not all(flag((nblk, j)) >= j + 1 for j in range(nblk - 1)):
                return False
            if not all(flag(("inv", j)) >= 1 for j in range(nblk - 1)):
                return False
            t = ws[ld + 2, :B * nblk].copy()
            t[B * (nblk - 1):] = st["ylast"]
            x = np.zeros(B * nblk)
            # row J: x_J = M_J t_J - P_J x_{J+1}, t_J holding every term
            # but x_{J+1}'s; x_{J+1}'s terms of the rows above J come off
            # in the same step
            for J in range(nblk - 1, -1, -1):
                xJ = Ms[J] @ t[B * J:B * J + B]
                if J + 1 < nblk:
                    x1 = x[B * (J + 1):B * (J + 2)]
                    xJ = xJ - Ps[J] @ x1
                    for I in range(J):
                        t[B * I:B * I + B] -= ws[upper(J + 1, I)].T @ x1
                x[B * J:B * J + B] = xJ
            st["x"] = x
            st["phase"] = "done"
            return True
        return False

    pc = [0] * len(lists)
    while True:
        progress = False
        for c in rng.permutation(len(lists) + 1):
            if c == len(lists):
                if st["phase"] != "done" and chain_step():
                    progress = True
            elif pc[c] < len(lists[c]) and ready(lists[c][pc[c]]):
                execute(lists[c][pc[c]])
                pc[c] += 1
                progress = True
        if st["phase"] == "done" and all(pc[c] == len(lists[c]) for c in range(len(lists))):
            break
        assert progress, f"deadlock at n={n}, C={C}: worker positions {pc}, chain step {st['k']}"
    x = st["x"][:n]
    ref = np.linalg.solve(A, b)
    return np.abs(x - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("n", [1, 5, 16, 17, 32, 48, 100, 168, 228, 256, 300, 384])
@pytest.mark.parametrize("C", [16, 8, 4])
def test_schedule_is_complete_deadlock_free_and_solves(n, C):
    for seed in range(4):
        assert emulate(n, C, seed) < 1e-10


def emulate_backward(nblk, seed):
    """The chain CTA's backward solve as the kernel runs it: warp 0 (x_J =
    v_J - P_J x_{J+1}), warp 4 (v_J = M_J t_J once row J is ready) and six
    helper warps (helper h owns the rows I = h mod 6 and applies x_K's terms
    L_KI^T x_K as x_K appears, K descending, row K-2 first, then marks row
    K-2 ready).  The warps step in random interleavings, each waiting on the
    counters the kernel waits on, and x must equal the triangular solve."""
    rng = np.random.default_rng(seed)
    n = B * nblk
    Lf = np.tril(rng.standard_normal((n, n)) * 0.3, -1) + np.eye(n)
    z = rng.standard_normal(n)
    blk = lambda a, i, j: a[B * i:B * i + B, B * j:B * j + B]
    Ms = [np.linalg.inv(blk(Lf, J, J)).T for J in range(nblk)]
    Ps = [Ms[J] @ blk(Lf, J + 1, J).T if J + 1 < nblk else None for J in range(nblk)]
    t = z.copy()
    xs = np.full(n, np.nan)
    cnt = {"x": 0, "v": 0}
    ready = [False] * nblk
    H = 6

    def warp0():
        for J in range(nblk - 1, -1, -1):
            y = Ps[J] @ xs[B * (J + 1):B * (J + 2)] if J + 1 < nblk else 0.0
            yield True
            while cnt["v"] < nblk - J:
                yield False
            xs[B * J:B * J + B] = t[B * J:B * J + B] - y
            cnt["x"] = nblk - J
            yield True

    def warp4():
        for J in range(nblk - 1, -1, -1):
            while J + 2 < nblk and not ready[J]:
                yield False
            t[B * J:B * J + B] = Ms[J] @ t[B * J:B * J + B]
            cnt["v"] = nblk - J
            yield True

    def helper(h):
        for K in range(nblk - 1, 1, -1):
            top = K - 2
            if top < h:
                continue
            while cnt["x"] < nblk - K:
                yield False
            x_k = xs[B * K:B * K + B].copy()
            assert not np.isnan(x_k).any()
            for I in range(top - (top - h) % H, -1, -H):
                t[B * I:B * I + B] -= blk(Lf, K, I).T @ x_k
                if I == top:
                    ready[I] = True
                yield True

    agents = [warp0(), warp4()] + [helper(h) for h in range(H)]
    alive = [True] * len(agents)
    while any(alive):
        progress = False
        for a in rng.permutation(len(agents)):
            if alive[a]:
                try:
                    progress |= next(agents[a])
                except StopIteration:
                    alive[a] = False
                    progress = True
        assert progress, f"backward solve deadlock at nblk={nblk}"
    ref = np.linalg.solve(Lf.T, z)
    return np.abs(xs - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("nblk", [1, 2, 3, 4, 7, 11, 17, 24])
def test_backward_dataflow_is_deadlock_free_and_solves(nblk):
    for seed in range(4):
        assert emulate_backward(nblk, seed) < 1e-9
