"""Device-resident 2-bit reference (minibwa's l2b layout): the oracle's window decoding
(l2b_getseq, l2b_meth_convert, in-place reversal) agrees with an independent numpy decode."""
import numpy as np


def test_oracle_window_decoding_matches_numpy(built):
    from minibwa_gb300 import synth
    from oracle import oracle as O
    r = synth.Reference2b([5000, 777, 12345, 31], n_runs=40, run_max=300)
    rng = np.random.default_rng(1)
    for it in range(500):
        k = int(rng.integers(0, len(r.ctg_len)))
        L = min(int(rng.integers(0, 600)), int(r.ctg_len[k]))
        st = int(rng.integers(0, int(r.ctg_len[k]) - L + 1))
        fl = int(rng.choice([0, 1, 2, 3, 4, 5]))
        assert np.array_equal(O.l2b_getseq(r, k, st, L, fl), r.window(k, st, L, fl)), (it, k, st, L, fl)
