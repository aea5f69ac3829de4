"""Host logic of the autotuner (no GPU): the shapes it offers and how cached
choices are named and replayed into a context."""

import json

import stntt_gb300 as st
from stntt_gb300 import tune


def test_batched_candidates():
    assert tune.batched_candidates(12) == [[12]]
    c13 = tune.batched_candidates(13)
    assert [13] in c13 and [4, 9] in c13 and [9, 4] in c13
    c18 = tune.batched_candidates(18)
    assert all(len(s) == 2 and sum(s) == 18 and all(4 <= x <= 13 for x in s) for s in c18)
    assert [7, 11] in c18 and [18] not in c18


def test_plan_candidates_offer_eight_element_tiles():
    shapes = list(tune.candidates(st.FIELD_GL64, 20))
    assert any(logs == [10, 10] and es == [8, 8] for logs, es, _ in shapes)
    assert any(logs == [10, 10] and es == [16, 16] for logs, es, _ in shapes)
    # 8 elements per thread only where every pass is 2^7..2^11 points
    assert not any(8 in es and any(lg < 7 or lg > 11 for lg in logs) for logs, es, _ in shapes)
    shapes24 = list(tune.candidates(st.FIELD_GL64, 24))
    assert any(logs == [8, 8, 8] and es == [8, 8, 8] for logs, es, _ in shapes24)
    assert not any(logs == [12, 12] and 8 in es for logs, es, _ in shapes24)


class _FakeCtx:
    device = 0

    def __init__(self):
        self.calls = []

    def set_plan(self, field, log_n, logs, elems=None, cols=None, small=False, batched=False):
        self.calls.append((field, log_n, list(logs), small, batched))


def test_cache_names_and_replay(tmp_path, monkeypatch):
    key = "TEST GPU|7|13000|10.3"
    monkeypatch.setattr(tune, "_key", lambda device: key)
    monkeypatch.setattr(tune, "PACKAGED", tmp_path / "none.json")
    cache = tmp_path / "plans.json"
    ctx = _FakeCtx()
    tune.record(ctx, st.FIELD_GL64, 18, {"logs": [7, 11], "E": [16, 16], "C": [0, 0], "us": 1.0, "batch": 128,
                                         "batched": True}, cache)
    tune.record(ctx, st.FIELD_U32, 20, {"logs": [10, 10], "E": [8, 8], "C": [4, 4], "us": 2.0, "batch": 1}, cache)
    tune.record(ctx, st.FIELD_GL64, 24, {"logs": [8, 8, 8], "E": [16] * 3, "C": [16, 16, 4], "us": 3.0, "batch": 1},
                cache)
    names = set(json.loads(cache.read_text())[key])
    assert names == {"gl64:18:batch", "u32:20:b1", "gl64:24"}
    assert tune.apply_cache(ctx, cache) == 3
    got = {(f, lg): (small, batched) for f, lg, _, small, batched in ctx.calls}
    assert got[(st.FIELD_GL64, 18)] == (False, True)
    assert got[(st.FIELD_U32, 20)] == (True, False)
    assert got[(st.FIELD_GL64, 24)] == (False, False)


def test_packaged_plans_parse():
    plans = json.loads(tune.PACKAGED.read_text())
    for cls, entries in plans.items():
        assert cls.count("|") == 1
        for name, e in entries.items():
            parts = name.split(":")
            assert parts[0] in ("gl64", "u32") and len(parts) in (2, 3)
            assert sum(e["logs"]) == int(parts[1])
            assert len(e["logs"]) == len(e["E"]) == len(e["C"])
            if len(parts) == 3:
                assert parts[2] in ("b1", "batch")
            # what the library accepts (a rejected entry would make every Context fail)
            assert 1 <= len(e["logs"]) <= 3 and all(1 <= lg <= 13 for lg in e["logs"])
            assert all((x & ~(st.PASS_VEC | st.PASS_CLUSTER)) in (0, 4, 8, 16, 32) for x in e["E"])
            if any(x & st.PASS_VEC for x in e["E"]):  # the vector-lines build: 8 or 16 points per line
                assert all((x & ~(st.PASS_VEC | st.PASS_CLUSTER)) in (0, 4, 8, 16) for x in e["E"]), name
                assert len(e["logs"]) > 1, name
            elif 8 in e["E"]:
                assert all(7 <= lg <= 11 for lg in e["logs"]), name
            if name.endswith(":batch"):
                assert len(e["logs"]) <= 2 and all(lg >= 4 for lg in e["logs"]), name
                if len(e["logs"]) == 2:
                    assert int(parts[1]) >= 13, name


def test_plan_candidates_offer_vector_lines_build():
    """--vec adds the vector-lines build (STNTT_PASS_VEC) of two- and
    three-pass splits with 2^7..2^10-point passes: 8 or 16 points per line, 4
    or 8 line groups."""
    from stntt_gb300 import tune

    cands = list(tune.candidates(st.FIELD_U32, 26, vec=True))
    vec = [c for c in cands if any(e & st.PASS_VEC for e in c[1]) and not any(e & st.PASS_CLUSTER for e in c[1])]
    assert ([9, 9, 8], [8 | st.PASS_VEC, 8 | st.PASS_VEC, 16 | st.PASS_VEC], [32, 32, 32]) in vec
    assert all(len(logs) in (2, 3) and all(7 <= lg <= 10 for lg in logs) and cols[0] in (16, 32)
               for logs, _, cols in vec if max(logs) <= 10)
    # wide two-pass tiles (2^11, 2^12 points): 1, 2 or 4 line groups within 512 threads
    wide = [c for c in vec if max(c[0]) > 10]
    assert all(len(logs) == 2 and all(c in (4, 8, 16) for c, lg in zip(cols, logs) if lg > 10)
               for logs, _, cols in wide)
    wide22 = [c for c in tune.candidates(st.FIELD_U32, 22, vec=True)
              if any(e & st.PASS_VEC for e in c[1]) and not any(e & st.PASS_CLUSTER for e in c[1]) and max(c[0]) > 10]
    assert ([11, 11], [8 | st.PASS_VEC] * 2, [4, 4]) in wide22  # one line group: more, narrower CTAs
    assert ([13, 13], [16 | st.PASS_VEC] * 2, [8, 8]) not in vec
    assert any(len(logs) == 2 for logs, es, _ in tune.candidates(st.FIELD_GL64, 20, vec=True)
               if any(e & st.PASS_VEC for e in es))
    gl = [c for c in tune.candidates(st.FIELD_GL64, 24, vec=True)
          if any(e & st.PASS_VEC for e in c[1]) and not any(e & st.PASS_CLUSTER for e in c[1])]
    assert gl and all(cols[0] in (8, 16) for logs, _, cols in gl if max(logs) <= 10)
    assert ([12, 12], [16 | st.PASS_VEC] * 2, [4, 4]) in gl  # two HBM passes at 2^24
    # at most 512 threads for the wide tiles: 2^12 points at 8 per line only with one line group
    assert all(cols[0] == 2 for logs, es, cols in gl if logs == [12, 12] and (es[0] & 0xff) == 8)
    assert not any(e & st.PASS_VEC for c in tune.candidates(st.FIELD_GL64, 24) for e in c[1])


def test_plan_candidates_offer_cluster_passes():
    """--vec also offers two-pass splits whose 2^11..2^13-point passes run in
    the vector-lines cluster build (STNTT_PASS_CLUSTER)."""
    cl = st.PASS_CLUSTER
    u = [c for c in tune.candidates(st.FIELD_U32, 26, vec=True) if any(e & cl for e in c[1])]
    assert ([13, 13], [8 | st.PASS_VEC | cl] * 2, [16, 16]) in u
    assert ([13, 13], [8 | st.PASS_VEC | cl] * 2, [32, 32]) in u  # 1024 threads x 64 registers
    g = [c for c in tune.candidates(st.FIELD_GL64, 24, vec=True) if any(e & cl for e in c[1])]
    assert ([12, 12], [8 | st.PASS_VEC | cl] * 2, [8, 8]) in g
    assert not any(logs == [13, 13] and cols == [16, 16] for logs, _, cols in
                   (c for c in tune.candidates(st.FIELD_GL64, 26, vec=True) if any(e & cl for e in c[1])))
    mixed = [c for c in tune.candidates(st.FIELD_GL64, 20, vec=True) if any(e & cl for e in c[1])]
    assert ([11, 9], [8 | st.PASS_VEC | cl, 8 | st.PASS_VEC], [8, 8]) in mixed
    assert all(len(logs) == 2 for logs, _, _ in u + g + mixed)


def test_verify_top_reranks_by_step_time():
    """--verify: the k fastest forward-only candidates are re-timed as forward
    + inverse steps and ranked by that time; the others are not timed again."""
    results = [{"logs": [10, 10], "us": 29.5}, {"logs": [11, 9], "us": 29.6}, {"logs": [9, 11], "us": 30.5},
               {"logs": [12, 8], "us": 40.0}]
    step = {(10, 10): 67.5, (11, 9): 60.9, (9, 11): 62.0}
    timed = []

    def step_us(r):
        timed.append(tuple(r["logs"]))
        return step[tuple(r["logs"])]

    ranked = tune.verify_top(results, 3, step_us)
    assert [r["logs"] for r in ranked] == [[11, 9], [9, 11], [10, 10]]
    assert ranked[0]["step_us"] == 60.9
    assert sorted(timed) == sorted(step) and "step_us" not in results[3]


def test_time_plan_step_orchestration(monkeypatch):
    """_time_plan's call sequence, with torch.cuda faked on the CPU: a small
    call is captured as one graph per direction and each timed step replays
    the forward graph then (inverse_too) the inverse one; a large call runs
    the C-ABI calls directly."""
    import contextlib

    import torch

    log = []

    class _Stream:
        cuda_stream = 1234

        def __init__(self, device=None):
            pass

        def synchronize(self):
            log.append("sync")

    class _Graph:
        n = 0

        def __init__(self):
            _Graph.n += 1
            self.id = _Graph.n

        def replay(self):
            log.append(f"replay{self.id}")

    capturing = []

    @contextlib.contextmanager
    def _graph(g, stream=None, capture_error_mode=None):
        capturing.append(g.id)
        yield
        capturing.pop()

    class _Event:
        def __init__(self, enable_timing=False):
            pass

        def record(self, stream=None):
            log.append("event")

        def elapsed_time(self, other):
            return 0.01

    monkeypatch.setattr(torch.cuda, "Stream", _Stream)
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(torch.cuda, "CUDAGraph", _Graph)
    monkeypatch.setattr(torch.cuda, "graph", _graph)
    monkeypatch.setattr(torch.cuda, "Event", _Event)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a: None)

    class _Ctx:
        def ntt_gl64(self, data, log_n, batch, inverse=False, stream=None):
            assert stream == 1234
            log.append(("inv" if inverse else "fwd") + (f"@g{capturing[-1]}" if capturing else ""))

    class _Data:
        device = "cpu"

    class _Flush:
        def zero_(self):
            log.append("flush")

    us = tune._time_plan(_Ctx(), st.FIELD_GL64, 20, _Data(), 0, 0, 1, 2, _Flush(), inverse_too=True)
    assert abs(us - 10.0) < 1e-9
    g1, g2 = _Graph.n - 1, _Graph.n
    assert log[:5] == ["fwd", "inv", "sync", f"fwd@g{g1}", f"inv@g{g2}"]
    timed = log[7:]  # after the warm-up replay of both graphs
    assert timed == ["flush", "event", f"replay{g1}", f"replay{g2}", "event"] * 2
    log.clear()
    tune._time_plan(_Ctx(), st.FIELD_GL64, 22, _Data(), 0, 0, 1, 1, _Flush())
    assert log == ["fwd", "sync", "fwd", "flush", "event", "fwd", "event"]
