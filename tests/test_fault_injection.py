"""Host-side fault injection (no GPU): the Python front end over a fake C-ABI
library whose entry points return injected error codes.  Every error becomes an
EngineError carrying the status code and the library's thread-local message,
no output is returned, and the engine stays usable for the next call."""
import numpy as np
import pytest

from contrafold_gpu_gb300 import engine as E


class FakeLib:
    """The subset of the C-ABI the batch calls use; `fail` maps entry point ->
    status code (absent = CF_OK)."""

    def __init__(self, fail):
        self.fail = dict(fail)
        self.calls = []
        self.destroyed = 0

    def cf_last_error(self):
        return b"injected failure"

    def cf_engine_destroy(self, h):
        self.destroyed += 1

    def __getattr__(self, name):
        if not name.startswith("cf_"):
            raise AttributeError(name)

        def call(*args):
            self.calls.append(name)
            if name == "cf_engine_create":
                args[-1]._obj.value = 1   # a non-null handle
            return self.fail.get(name, E.CF_OK)
        return call


def _engine(monkeypatch, P, fail):
    lib = FakeLib(fail)
    monkeypatch.setattr(E, "load_library", lambda *a, **k: lib)
    return E.Engine(P), lib


@pytest.mark.parametrize("code", [E.CF_EINVAL, E.CF_ENOMEM, E.CF_ETIMEOUT, E.CF_ECUDA, E.CF_EDEVICE])
def test_injected_status_raises_engine_error(monkeypatch, P, code):
    eng, lib = _engine(monkeypatch, P, {"cf_mea": code, "cf_logz": code, "cf_bpp": code})
    B = E.Batch(["GGGGAAAACCCC", "ACGU"])
    for call in (lambda: eng.mea(B, 6.0), lambda: eng.logz(B), lambda: eng.bpp(B)):
        with pytest.raises(E.EngineError) as ei:
            call()
        assert ei.value.code == code
        assert "injected failure" in str(ei.value)
    # an entry point that does not fail still works on the same engine (the
    # fake writes nothing, so the structures are the right lengths of NULs)
    assert [len(s) for s in eng.mfe(B)] == [12, 4]
    assert lib.calls.count("cf_mea") == 1 and "cf_mfe" in lib.calls
    eng.close()
    assert lib.destroyed == 1


def test_engine_create_failure(monkeypatch, P):
    lib = FakeLib({"cf_engine_create": E.CF_ECUDA})
    monkeypatch.setattr(E, "load_library", lambda *a, **k: lib)
    with pytest.raises(E.EngineError) as ei:
        E.Engine(P)
    assert ei.value.code == E.CF_ECUDA


def test_front_end_propagates(monkeypatch, P):
    """The reference-shaped API (logZ_batch, mea_batch) surfaces the error."""
    from contrafold_gpu_gb300 import gpu
    eng, _ = _engine(monkeypatch, P, {"cf_logz": E.CF_ENOMEM, "cf_mea": E.CF_EDEVICE})
    monkeypatch.setattr(gpu, "engine_for", lambda *a, **k: eng)
    with pytest.raises(E.EngineError) as ei:
        gpu.logZ_batch(["ACGU"], P)
    assert ei.value.code == E.CF_ENOMEM
    with pytest.raises(E.EngineError) as ei:
        gpu.mea_batch(["ACGU"], P, forced_list=[np.array([0, 1, 0, 0], np.int8)])
    assert ei.value.code == E.CF_EDEVICE


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No silent fallback: without the built library the engine refuses to start."""
    monkeypatch.setattr(E, "_lib", None)
    with pytest.raises(E.EngineError) as ei:
        E.load_library(str(tmp_path / "missing.so"))
    assert ei.value.code == E.CF_ECUDA and "not built" in str(ei.value)
