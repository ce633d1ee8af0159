"""Host logic of the FP32 factorization autotuner (boltzmann_gb300.autotune) with the timing
and the device name stubbed: no GPU needed."""
import json

from boltzmann_gb300 import autotune


def test_fastest_candidate_is_kept_and_cached(tmp_path, monkeypatch):
    monkeypatch.setenv("BOLTZMANN_GB300_CACHE", str(tmp_path))
    monkeypatch.setattr(autotune, "_mem", {})
    monkeypatch.setattr(autotune, "_key", lambda N, device: "fake-gpu|N=%d" % N)
    fake_ms = {2: 3.0, 4: 2.5, 5: 2.8, 3: 4.0, 1: 9.0}
    calls = []

    def fake_time(N, kernel, **kw):
        calls.append((N, kernel))
        return fake_ms[kernel]

    monkeypatch.setattr(autotune, "time_lu", fake_time)
    rec = autotune.tune_lu(385)
    assert rec["kernel"] == 4 and sorted(k for _, k in calls) == [1, 2, 3, 4, 5]
    data = json.load(open(tmp_path / "lu_autotune.json"))
    assert data["fake-gpu|N=385"]["kernel"] == 4
    # sizes above 512: the right-looking kernel is the only candidate
    assert autotune.tune_lu(1025)["kernel"] == 1
    # a fresh process reads the disk cache instead of timing again
    monkeypatch.setattr(autotune, "_mem", {})
    calls.clear()
    assert autotune.lu_kernel_for(385) == 4 and not calls
