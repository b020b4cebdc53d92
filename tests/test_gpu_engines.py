"""Several engines in one process.  A kernel's dynamic shared-memory limit is
an attribute of the function, shared by every engine: an engine that needs
little must not lower the limit another engine's launches rely on."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_engines_do_not_lower_each_others_shared_memory(P):
    from contrafold_gpu_gb300.engine import Batch, Engine
    rng = np.random.default_rng(51)
    seqs = ["".join(rng.choice(list("ACGU"), size=560)) for _ in range(32)]
    big = Batch(seqs)
    a = Engine(P)
    a.set_schedule("group")
    a.set_group(32)                  # the codes of 32 sequences of 560 nt in one CTA: above the 48 KB default
    want = a.mea(big, 6.0)
    b = Engine(P)                    # a second engine with small launches only
    assert len(b.mea(Batch(["GGGGAAAACCCC"]), 6.0)[0]) == 12
    assert a.mea(big, 6.0) == want   # engine a's large launch still goes through
    a.set_schedule("group")
    a.set_group(0)
    assert a.mea(big, 6.0) == want
    a.close()
    b.close()


def test_shared_device_and_priority_keep_results(P):
    """An engine in shared-device mode (no 512-thread CTAs, no clusters) and at
    either stream priority folds exactly what the default engine folds."""
    from contrafold_gpu_gb300.engine import Batch, Engine
    rng = np.random.default_rng(52)
    seqs = ["".join(rng.choice(list("ACGU"), size=int(L))) for L in (520, 560, 600, 150)]
    masks = [(rng.random(len(s)) < 0.1).astype(np.int8) for s in seqs]
    eng = Engine(P)
    try:
        for B in (Batch(seqs[:3], masks[:3]), Batch(seqs, masks)):   # all >= 512 nt (cluster row), and mixed
            want = (eng.mea(B, 6.0), eng.logz(B).tobytes(), eng.sample(B, 5, seed=3))
            eng.set_shared(True)
            for high in (True, False, True):
                eng.set_priority(high)
                assert (eng.mea(B, 6.0), eng.logz(B).tobytes(), eng.sample(B, 5, seed=3)) == want
            eng.set_priority(False)
            eng.set_shared(False)
    finally:
        eng.close()
