"""The surrogate recipe's selection logic on the CPU, with the GPU parts
(pair generation, training, tissue validation) replaced by stand-ins: every
candidate is trained on the same pairs, scored on the validation tissue, the
least biased one is kept and saved with all scores, and the others are
released."""
import numpy as np
import pytest


def test_train_default_keeps_least_biased_candidate(monkeypatch, tmp_path):
    torch = pytest.importorskip("torch")
    from lqt1_gb300 import surrogate as S
    biases = {1: 0.5, 2: -0.1, 3: 0.3, 4: -0.2}
    closed, saved, gen_calls, trained = [], {}, [], []

    class FakeMlp:
        def __init__(self, seed=0, stream=None):
            self.seed = seed
            self.nsub = 5

        def set_norm(self, *a):
            pass

        def set_bounds(self, b):
            pass

        def close(self):
            closed.append(self.seed)

    def fake_generate(**kw):
        gen_calls.append(kw)
        return torch.zeros(64, 44), torch.zeros(64, 38)

    def fake_train(m, X, D, **kw):
        trained.append((m.seed, kw["seed"], kw["oversample"], id(X)))
        return dict(rmse=np.full(38, 0.1), zero_rmse=np.ones(38), n=10), [(0, 1.0)]

    monkeypatch.setattr(S, "Mlp", FakeMlp)
    monkeypatch.setattr(S, "generate", fake_generate)
    monkeypatch.setattr(S, "fit_norm", lambda X, D: (np.zeros(48), np.ones(48), np.ones(48)))
    monkeypatch.setattr(S, "fit_bounds", lambda D, osc: np.ones(48))
    monkeypatch.setattr(S, "train", fake_train)
    monkeypatch.setattr(S, "validate_tissue",
                        lambda m, ref=None: (biases[m.seed], abs(biases[m.seed]) + 0.05, "ref"))
    monkeypatch.setattr(S, "save", lambda m, out, meta: saved.update(m=m, out=out, meta=meta))
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a: None)

    m, meta = S.train_default(str(tmp_path / "w.npz"), seed=1, select=4, nsub=10, log=lambda s: None)
    assert len(gen_calls) == 1 and gen_calls[0]["nsub"] == 10          # one set of pairs for all
    assert [t[0] for t in trained] == [1, 2, 3, 4] and len({t[3] for t in trained}) == 1
    assert all(t[2] == 4 for t in trained)                              # phase-3 oversampling by default
    assert m.seed == 2 and meta["seed"] == 2 and saved["m"] is m and m.nsub == 10
    assert [c["seed"] for c in meta["candidates"]] == [1, 2, 3, 4]
    assert [c["apd_bias_ms"] for c in meta["candidates"]] == [0.5, -0.1, 0.3, -0.2]
    assert sorted(closed) == [1, 3, 4]                                  # every other candidate released
    assert meta["macro_steps"] == 10 and meta["data_seed"] == 1
