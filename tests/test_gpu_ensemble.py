"""Batched ensemble (hosnwt_advance_many): independent tanks advanced
together give the same states, to rounding, as the same tanks advanced
one by one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_advance_many_matches_single(lib):
    import hosnwt
    import workloads
    specs = workloads.ensemble(n_tanks=4, seed=3, T_stop=4.0)
    for s in specs:  # keep the test small: shrink the grids
        s["n1"] = min(s["n1"], 257)
        s["n3"] = 17
    def make():
        return [hosnwt.Tank(s["inp"], s["n1"], 1, s["n3"], s["mHOS"], s["p1"], 1, probes=s["probes"])
                for s in specs]
    single = make()
    batch = make()
    tn = []
    for t in single:
        inf = t.info()
        T = 0.3 / inf["Tscale"]
        t.advance(T, inf["delt"])
        tn.append(T)
    hr = hosnwt.advance_many(batch, tn, [t.info()["delt"] for t in batch])
    assert np.all(hr > 0)
    for a, b in zip(single, batch):
        ea, pa, _ = a.get_state()
        eb, pb, _ = b.get_state()
        # single advance runs the step control on the device, advance_many on
        # the host: the two evaluate pow() of the step correction on different
        # processors, so the states agree to rounding, not bit for bit
        assert abs(a.info()["time_cur"] - b.info()["time_cur"]) <= 1e-12
        assert np.max(np.abs(ea - eb)) <= 1e-10 * np.max(np.abs(eb))
        assert np.max(np.abs(pa - pb)) <= 1e-10 * np.max(np.abs(pb))
        assert np.max(np.abs(ea)) > 0.0
