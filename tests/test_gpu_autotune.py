"""The autotuner times every eligible thread-group shape and lane width per n_col_ class and
installs the fastest; results under the tuned choices stay bit-exact."""
import numpy as np
import pytest

from conftest import EXT_FIELDS

pytestmark = pytest.mark.gpu


def test_tune_and_apply_keep_results(built):
    from minibwa_gb300 import Context, autotune, synth
    p = synth.config1(6000, seed=91)
    ctx = Context(0)
    before, bcig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    table = autotune.tune_ext(ctx, p, sample=512, reps=2, min_class=64)
    assert table, "no n_col_ class was tuned"
    shp = autotune.shapes()
    for (dual, mode, nc), (g, k, w16, per_choice) in table.items():
        assert g * k >= 4 * nc and (g, k) in shp and w16 in (0, 1)
        assert (g, k, w16) == min(per_choice, key=per_choice.get)  # the fastest choice was installed
        assert {w for (_, _, w) in per_choice} == {0, 1}  # both lane widths were timed
    autotune.apply(table)
    after, acig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    for f in EXT_FIELDS:
        assert np.array_equal(before[f], after[f]), f
    for i in range(0, len(p), 37):
        o, n, o2 = int(before["cigar_off"][i]), int(before["n_cigar"][i]), int(after["cigar_off"][i])
        assert np.array_equal(bcig[o:o + n], acig[o2:o2 + n])
    autotune.reset(table)
    ctx.close()
