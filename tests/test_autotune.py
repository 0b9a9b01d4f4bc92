"""Batch-schedule autotuner: the candidate wave sizes (host logic) and its cache."""
import json

from quantum_transport_gb300 import autotune


def test_candidates_span_two_to_eight_items_per_sm_and_the_whole_call():
    c = autotune.candidates(1024, nk=16, sms=152)
    assert c == [304, 448, 608, 752, 912, 1024]
    assert all(p % 16 == 0 for p in c)


def test_candidates_never_exceed_the_call_or_drop_below_one_energy():
    assert autotune.candidates(100, nk=1, sms=152) == [100]
    assert autotune.candidates(5, nk=8, sms=152) == [8]


class _FakeCtx:
    def __init__(self):
        self.wave = None

    def set_wave_points(self, p):
        self.wave = p


def test_cached_choice_is_reused_without_timing(tmp_path, monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda i: "GPU-X")
    cache = tmp_path / "waves.json"
    cache.write_text(json.dumps({"GPU-X|chain": {"best": 912, "ms": {"608": 2.0, "912": 1.5}}}))
    ctx = _FakeCtx()
    calls = []
    best, ms = autotune.tune_wave(ctx, lambda: calls.append(1), 1024, nk=16, cache=str(cache),
                                  key="chain")
    assert best == 912 and ctx.wave == 912 and not calls and ms == {608: 2.0, 912: 1.5}
