"""The autotuner's search logic (matmri_gb300/autotune.py) on a fake operator with a synthetic
cost model: no GPU.  The GPU side (timing the real normal operator) runs in bench.py."""
import itertools

from matmri_gb300 import autotune as at


class FakeOp:
    """Records settings; the 'time' of a setting comes from a cost function of the knobs."""

    def __init__(self, start, C=32):
        self.t = dict(zip(at.KNOBS, start))
        self.C = C
        self.seen = []

    def get_tuning(self):
        return tuple(self.t[k] for k in at.KNOBS)

    def set_tuning(self, **kw):
        self.t.update({k: v for k, v in kw.items() if v})
        self.seen.append(self.get_tuning())


def test_search_finds_a_joint_optimum_coordinate_steps_miss():
    # tile 16 only pays off together with 4 coils per CTA (and stencil mode 2 is always slower):
    # a pure coordinate descent from (32, 2) stays there
    def cost(t):
        base = 1.0 + 0.1 * (t["normal_mode"] == 2) + 0.01 * abs(t["item"] - 256) / 256
        pair = {(32, 2): 0.0, (16, 4): -0.05}.get((t["tile"], t["coil_group"]), 0.08)
        return base + pair + 0.02 * (t["coil_chunk"] != 32) + 0.01 * (t["fft_lines"] != 4)

    op = FakeOp((8, 32, 4, 64, 8, 2))
    knobs, ms = at.search(op, lambda: cost(op.t))
    assert (knobs["tile"], knobs["coil_group"], knobs["normal_mode"]) == (16, 4, 1)
    assert knobs["coil_chunk"] == 32 and knobs["item"] == 256 and knobs["fft_lines"] == 4
    assert abs(ms - cost(knobs)) < 1e-12
    assert op.get_tuning() == tuple(knobs[k] for k in at.KNOBS)     # left at the optimum


def test_search_visits_every_tile_coil_group_pair_and_both_modes():
    op = FakeOp((16, 32, 2, 128, 4, 1), C=16)
    at.search(op, lambda: 1.0)
    pairs = {(s[1], s[2]) for s in op.seen}
    assert pairs >= set(itertools.product(at.SPACE["tile"], at.SPACE["coil_group"]))
    assert {s[5] for s in op.seen} >= set(at.SPACE["normal_mode"])
    assert max(s[0] for s in op.seen) <= 16      # no coil chunk above the operator's coils
