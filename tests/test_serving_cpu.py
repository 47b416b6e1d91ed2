"""Host side of serving, without a GPU: the seeded mixed job stream follows
its definition (lattice, L, species, shells, V range, kinds) and is the same
for the same master seed."""
import numpy as np

from brawl_gb300 import RY_TO_EV
from brawl_gb300 import serving as S


def test_stream_is_seeded_and_within_its_ranges():
    a = S.stream_jobs(300, master_seed=11)
    b = S.stream_jobs(300, master_seed=11)
    kinds = set()
    for ja, jb in zip(a, b):
        assert ja["seed"] == jb["seed"] and ja["kind"] == jb["kind"] and np.array_equal(ja["V"], jb["V"])
        assert ja["lattice"] in ("fcc", "bcc") and 6 <= ja["L"] <= 32
        s = ja["setup"]
        assert 2 <= s.n_species <= 5 and 2 <= s.interaction_range <= 6
        assert np.abs(ja["V"]).max() <= 0.05 / RY_TO_EV + 1e-15
        assert np.array_equal(ja["V"], ja["V"].transpose(1, 0, 2))       # symmetric in the species
        assert ja["numbers"].sum() == ja["N"] and (ja["numbers"] >= 1).all()
        assert abs(ja["conc"][1:].sum() - 1.0) < 1e-12
        kinds.add(ja["kind"])
        if ja["kind"] == "anneal":
            assert 100 <= 4 * ja["sweeps_per_T"] <= 2000 + 3
        assert S.job_trials(ja) > 0
    assert kinds == {"anneal", "wl", "ns"}
    c = S.stream_jobs(300, master_seed=12)
    assert any(x["seed"] != y["seed"] for x, y in zip(a, c))
