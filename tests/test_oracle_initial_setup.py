"""initial_setup (src/initialise.F90:434-617) in the oracle against a
pure-Python restatement of the reference's loop, on streams with a word
planted on the boundary of two species' intervals: every species whose
interval holds the draw and whose quota is open takes the site and uses up
one unit of its quota, the last one keeping it.  (With both quotas open the
configuration can never be completed and the reference's loop never ends;
that case is the device's error path, tested on the GPU.)"""
import numpy as np

from oracle import oracle as O


def _untemper(y):
    y ^= y >> 18
    y ^= (y << 15) & 0xEFC60000
    t = y
    for _ in range(5):
        t = y ^ ((t << 7) & 0x9D2C5680)
    y = t & 0xFFFFFFFF
    t = y
    for _ in range(3):
        t = y ^ (t >> 11)
    return t & 0xFFFFFFFF


def _restated(r, n, counts):
    """The reference's fcc loop: sites in z, y, x order; per site, draws until
    a species is written; every open species holding the draw is written in
    turn and uses up one unit of its quota."""
    ns = len(counts)
    conc = [0.0] + [float(np.float32(np.float32(c) / np.float32(4 * n ** 3))) for c in counts]
    lo = [sum(conc[:l]) for l in range(1, ns + 1)]
    hi = [sum(conc[:l + 1]) for l in range(1, ns + 1)]
    check = [0] * ns
    W = 2 * n
    cfg = np.zeros((W, W, W), dtype=np.int8)   # [z, y, x]
    for z in range(W):
        for y in range(W):
            for x in range(W):
                if (x + y + z) % 2:
                    continue
                while cfg[z, y, x] == 0:
                    u = r.uniform()
                    for l in range(ns):
                        if lo[l] <= u <= hi[l] and check[l] < counts[l]:
                            cfg[z, y, x] = l + 1
                            check[l] += 1
    return cfg


def test_boundary_word_with_one_quota_full():
    V = np.zeros((2, 2, 1))
    mod = O.OracleModel("fcc", 2, 2, 2, V)
    counts = [1, 31]                       # species 1 holds [0, 2^27], species 2 [2^27, 2^32 - 1]
    base = O.OracleRng(4321).state_words()
    # species 1's one atom is drawn first, so the boundary word finds its
    # quota full; a boundary word drawn first would use up both quotas
    for plant in ([100, 1 << 27], [77, 99, 1 << 27, 1 << 27]):
        st = base.copy()
        for k, w in enumerate(plant):
            st[k] = _untemper(w)
        st[624] = 0
        a, b = O.OracleRng(1), O.OracleRng(1)
        a.set_state_words(st)
        b.set_state_words(st)
        cfg, _ = mod.initial_setup(a, np.array([0.0, 0.5, 0.5]), np.array(counts, dtype=np.int64))
        ref = _restated(b, 2, counts)
        assert np.array_equal(cfg.reshape(4, 4, 4), ref), plant
        assert a.u32() == b.u32()
