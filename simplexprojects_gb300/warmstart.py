"""Learned warm start: predict the optimal basis of perturbed LPs.

A family of LPs shares A (and the shapes m, n) and perturbs c and b (the
kind-3 workload).  The plain FP64 GPU solver produces the optimal bases of a
training set; a multilayer perceptron (hand-written BF16 tensor-core kernels
in libblpg, ``blpg_mlp_*``) learns to score every column for membership in
the optimal basis from the LP's normalised [c; b; family one-hot].  For a new
LP the m highest-scoring columns (``blpg_topm_hint``) become the basis hint
of the solver, which pivots them in and finishes by primal simplex, dual
simplex or a cost-shifted dual phase (see include/blpg.h, basis_hint).

Everything on the hot path (features, inference, top-m, solve) runs as
libblpg kernels on device-resident data; torch provides device buffers and
streams only.
"""
from __future__ import annotations

import ctypes as C
import json
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional

import numpy as np

from . import _native as N
from .lp import LPBatch


def _vp(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class MLP:
    """Owner of a blpg_mlp (parameters, optimizer state, activations)."""

    def __init__(self, d_in: int, d_out: int, hidden: int = 512, layers: int = 3,
                 max_batch: int = 512, seed: int = 1):
        self.L = N.lib()
        h = C.c_void_p()
        N.check(self.L.blpg_mlp_create(d_in, hidden, layers, d_out, max_batch, seed, C.byref(h)),
                "blpg_mlp_create")
        self.h = h
        a, b = C.c_int32(), C.c_int32()
        N.check(self.L.blpg_mlp_dims(h, C.byref(a), C.byref(b)), "blpg_mlp_dims")
        self.d_in, self.d_out, self.hidden, self.layers = d_in, d_out, hidden, layers
        self.d_in_pad, self.d_out_pad = a.value, b.value
        self.max_batch = max_batch

    def num_params(self) -> int:
        return int(self.L.blpg_mlp_num_params(self.h))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params(), np.float32)
        N.check(self.L.blpg_mlp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))),
                "blpg_mlp_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params()
        N.check(self.L.blpg_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))),
                "blpg_mlp_set_params")

    def train_step(self, X, Y, lr: float, stream=None) -> float:
        loss = C.c_float()
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        N.check(self.L.blpg_mlp_train_step(self.h, _vp(X), _vp(Y), X.shape[0], lr,
                                           C.byref(loss), s), "blpg_mlp_train_step")
        return loss.value

    def predict_launches(self, rows: int) -> int:
        """Kernels one predict() of `rows` rows launches: per chunk of at most
        max_batch rows, one BF16 conversion and layers + 1 GEMMs."""
        chunks = (rows + self.max_batch - 1) // self.max_batch
        return chunks * (self.layers + 2)

    def predict(self, X, out, stream=None) -> None:
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        N.check(self.L.blpg_mlp_predict(self.h, _vp(X), X.shape[0], _vp(out), s),
                "blpg_mlp_predict")

    def gradients(self, X, Y):
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_float()
        N.check(self.L.blpg_mlp_gradients(self.h, _vp(X), _vp(Y), X.shape[0],
                                          g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)),
                "blpg_mlp_gradients")
        return g, loss.value

    def close(self):
        if self.h:
            self.L.blpg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class TrainReport:
    epochs: int
    seconds: float
    losses: list = field(default_factory=list)
    train_lps: int = 0


class WarmStart:
    """The learned warm start for LPs of one shape (m rows, n columns) drawn
    from `families` families (kind-3 workload: m=174, n=142, 64 families)."""

    def __init__(self, m: int, n: int, families: int = 64, hidden: int = 512, layers: int = 3,
                 max_batch: int = 512, seed: int = 1, device: str = "cuda:0"):
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        self.m, self.n, self.F = m, n, families
        self.nf = n + m
        self.mlp = MLP(self.nf + families, self.nf, hidden, layers, max_batch, seed)
        self.mean = None
        self.std = None

    # ---- data -------------------------------------------------------------
    def fit_stats(self, batch: LPBatch) -> None:
        """Per-family, per-feature mean and std of [c; b] on the training set."""
        k = batch.count
        _, ob, oc = batch.offsets()
        feats = np.empty((k, self.nf), np.float64)
        for i in range(k):
            feats[i, :self.n] = batch.c[oc[i]:oc[i] + self.n]
            feats[i, self.n:] = batch.b[ob[i]:ob[i] + self.m]
        mean = np.zeros((self.F, self.nf))
        std = np.ones((self.F, self.nf))
        for f in range(self.F):
            sel = feats[batch.family == f]
            if len(sel):
                mean[f] = sel.mean(0)
                sd = sel.std(0)
                std[f] = np.where(sd > 1e-12, sd, 1.0)
        self.mean = self.torch.from_numpy(mean.astype(np.float32)).to(self.dev)
        self.std = self.torch.from_numpy(std.astype(np.float32)).to(self.dev)

    def device_inputs(self, batch: LPBatch):
        """Device copies of what the feature kernel reads (b, c, offsets, family)."""
        torch = self.torch
        _, ob, oc = batch.offsets()
        return dict(b=torch.from_numpy(batch.b).to(self.dev), c=torch.from_numpy(batch.c).to(self.dev),
                    ob=torch.from_numpy(np.ascontiguousarray(ob)).to(self.dev),
                    oc=torch.from_numpy(np.ascontiguousarray(oc)).to(self.dev),
                    fam=torch.from_numpy(batch.family.astype(np.int32)).to(self.dev),
                    count=batch.count)

    def features(self, d, out=None, stream=None):
        """Feature rows (count padded to 64) of a device batch (device_inputs)."""
        torch = self.torch
        rows = (d["count"] + 63) // 64 * 64
        if out is None:
            out = torch.zeros((rows, self.mlp.d_in_pad), dtype=torch.float32, device=self.dev)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        N.check(N.lib().blpg_features(d["count"], self.m, self.n, self.F, _vp(d["ob"]),
                                      _vp(d["oc"]), _vp(d["b"]), _vp(d["c"]), _vp(d["fam"]),
                                      _vp(self.mean), _vp(self.std), _vp(out),
                                      self.mlp.d_in_pad, s), "blpg_features")
        return out

    def labels(self, basis: np.ndarray, count: int):
        """0/1 rows: column j is basic in the LP's optimal basis."""
        Y = np.zeros(((count + 63) // 64 * 64, self.mlp.d_out_pad), np.float32)
        B = basis.reshape(count, self.m)
        Y[np.repeat(np.arange(count), self.m), B.ravel()] = 1.0
        return self.torch.from_numpy(Y).to(self.dev)

    # ---- training ---------------------------------------------------------
    def train(self, batch: LPBatch, basis: np.ndarray, epochs: int = 20, lr: float = 1e-3,
              batch_size: Optional[int] = None, seed: int = 0, log=None) -> TrainReport:
        """Fit the network on LPs with known optimal bases (packed m per LP)."""
        torch = self.torch
        bs = batch_size or self.mlp.max_batch
        bs = max(64, min(bs, batch.count // 64 * 64))
        t0 = time.perf_counter()
        self.fit_stats(batch)
        X = self.features(self.device_inputs(batch))
        Y = self.labels(basis, batch.count)
        k = batch.count
        steps = max(1, k // bs)
        rng = np.random.default_rng(seed)
        rep = TrainReport(epochs, 0.0, train_lps=k)
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(k)).to(self.dev)
            tot = 0.0
            for s in range(steps):
                idx = perm[s * bs:(s + 1) * bs]
                tot += self.mlp.train_step(X.index_select(0, idx).contiguous(),
                                           Y.index_select(0, idx).contiguous(), lr)
            rep.losses.append(tot / max(1, steps * bs * self.nf))
            if log:
                log(f"epoch {ep}: mean BCE {rep.losses[-1]:.4f}")
        torch.cuda.synchronize()
        rep.seconds = time.perf_counter() - t0
        return rep

    # ---- inference --------------------------------------------------------
    def hint_launches(self, count: int) -> int:
        """Kernels one predict_hint() over `count` LPs launches: features,
        the network, top-m."""
        return 1 + self.mlp.predict_launches((count + 63) // 64 * 64) + 1

    def predict_hint(self, d, m_dev, n_dev, offhint_dev, hint_out=None, stream=None,
                     scratch=None):
        """Basis hints (int32, packed m per LP) for a device batch."""
        torch = self.torch
        X = self.features(d, out=scratch.get("X") if scratch else None, stream=stream)
        rows = X.shape[0]
        logits = (scratch.get("logits") if scratch else None)
        if logits is None:
            logits = torch.empty((rows, self.mlp.d_out_pad), dtype=torch.float32, device=self.dev)
        self.mlp.predict(X, logits, stream)
        if hint_out is None:
            hint_out = torch.empty(d["count"] * self.m, dtype=torch.int32, device=self.dev)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        N.check(N.lib().blpg_topm_hint(_vp(logits), self.mlp.d_out_pad, d["count"], _vp(m_dev),
                                       _vp(n_dev), self.nf, _vp(offhint_dev), _vp(hint_out), s),
                "blpg_topm_hint")
        return hint_out

    def weights_launches(self, count: int) -> int:
        """Kernels one predict_weights() over `count` LPs launches."""
        return 1 + self.mlp.predict_launches((count + 63) // 64 * 64) + 1

    def predict_weights(self, d, m_dev, n_dev, offw_dev, w_out=None, stream=None, scratch=None,
                        beta: float = 1.0):
        """Steepest-edge score factors 1 + beta * p_j (p_j the network's
        probability that column j is basic), n + m per LP, for a device batch."""
        torch = self.torch
        X = self.features(d, out=scratch.get("X") if scratch else None, stream=stream)
        rows = X.shape[0]
        logits = (scratch.get("logits") if scratch else None)
        if logits is None:
            logits = torch.empty((rows, self.mlp.d_out_pad), dtype=torch.float32, device=self.dev)
        self.mlp.predict(X, logits, stream)
        if w_out is None:
            w_out = torch.empty(d["count"] * self.nf, dtype=torch.float32, device=self.dev)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        N.check(N.lib().blpg_price_weights(_vp(logits), self.mlp.d_out_pad, d["count"], _vp(m_dev),
                                           _vp(n_dev), self.nf, _vp(offw_dev), float(beta),
                                           _vp(w_out), s), "blpg_price_weights")
        return w_out

    # ---- checkpoints ------------------------------------------------------
    def save(self, path: str) -> None:
        """Parameters (binary FP32) and a JSON header with the dimensions and
        the feature statistics."""
        p = Path(path)
        params = self.mlp.get_params()
        head = dict(m=self.m, n=self.n, families=self.F, hidden=self.mlp.hidden,
                    layers=self.mlp.layers, num_params=int(params.size),
                    mean=self.mean.cpu().numpy().tolist(), std=self.std.cpu().numpy().tolist())
        p.with_suffix(".json").write_text(json.dumps(head))
        params.tofile(p.with_suffix(".bin"))

    @classmethod
    def load(cls, path: str, device: str = "cuda:0") -> "WarmStart":
        p = Path(path)
        head = json.loads(p.with_suffix(".json").read_text())
        ws = cls(head["m"], head["n"], head["families"], head["hidden"], head["layers"],
                 device=device)
        ws.mlp.set_params(np.fromfile(p.with_suffix(".bin"), dtype=np.float32))
        ws.mean = ws.torch.tensor(head["mean"], dtype=ws.torch.float32, device=ws.dev)
        ws.std = ws.torch.tensor(head["std"], dtype=ws.torch.float32, device=ws.dev)
        return ws


def basis_accuracy(pred: np.ndarray, truth: np.ndarray, m: int):
    """(mean fraction of predicted columns that are truly basic, fraction of
    LPs whose whole basis is predicted)."""
    P = pred.reshape(-1, m)
    T = truth.reshape(-1, m)
    hits = np.array([len(set(p) & set(t)) for p, t in zip(P, T)])
    return float(hits.mean() / m), float((hits == m).mean())


class LearnedSolver:
    """Solve batches of one LP shape with the learned warm start.

    Two ways of using the network:
      mode="guided" (default): the slack-basis primal simplex with
        steepest-edge pricing whose scores are multiplied by 1 + p_j, p_j
        the network's probability that column j is basic in the optimum;
      mode="crash": the m most probable columns as a basis hint, pivoted in
        and finished by primal, dual or cost-shifted dual simplex (cold
        solve as the fallback), with the plan's pricing (Dantzig unless
        ``pricing="steepest"`` is passed).

    ``run()`` enqueues features -> network -> weights or hint -> solve on
    device-resident data (the plan's CUDA graph for the solve);
    ``solve(batch)`` is the end-to-end call from host arrays (copies of A, b,
    c in, status / objective / pivots out): in guided mode one call of the C
    ABI's blpg_learned_solve, which runs the same kernels in the same order."""

    def __init__(self, ws: WarmStart, batch: LPBatch, precision: str = "fp32",
                 mode: str = "guided", beta: float = 1.0, **opts):
        import torch
        from .solver import DeviceBatch
        if mode not in ("guided", "crash"):
            raise ValueError("mode must be 'guided' or 'crash'")
        self.torch = torch
        self.ws = ws
        self.batch = batch
        self.mode = mode
        self.beta = beta
        if mode == "guided":
            opts["pricing"] = "steepest"
        self.db = DeviceBatch(batch, precision, device=str(ws.dev), **opts)
        self.d = ws.device_inputs(batch)
        # the feature kernel and the solver read the same b, c buffers
        self.d["b"], self.d["c"] = self.db.b, self.db.c
        k = batch.count
        self.m_dev = torch.from_numpy(batch.m).to(ws.dev)
        self.n_dev = torch.from_numpy(batch.n).to(ws.dev)
        offh = np.concatenate([[0], np.cumsum(batch.m.astype(np.int64))[:-1]]).astype(np.int64)
        self.offh_dev = torch.from_numpy(offh).to(ws.dev)
        nm = (batch.n + batch.m).astype(np.int64)
        offw = np.concatenate([[0], np.cumsum(nm)[:-1]]).astype(np.int64)
        self.offw_dev = torch.from_numpy(offw).to(ws.dev)
        self.hint = torch.empty(int(batch.m.sum()), dtype=torch.int32, device=ws.dev)
        self.weight = torch.empty(int(nm.sum()), dtype=torch.float32, device=ws.dev)
        rows = (k + 63) // 64 * 64
        self.opts = opts
        self.precision = precision
        self._cl = None  # the C ABI's blpg_learned, made at the first solve()
        self.scratch = dict(
            X=torch.zeros((rows, ws.mlp.d_in_pad), dtype=torch.float32, device=ws.dev),
            logits=torch.empty((rows, ws.mlp.d_out_pad), dtype=torch.float32, device=ws.dev))

    def predict(self, stream=None):
        if self.mode == "guided":
            return self.ws.predict_weights(self.d, self.m_dev, self.n_dev, self.offw_dev,
                                           self.weight, stream, self.scratch, self.beta)
        return self.ws.predict_hint(self.d, self.m_dev, self.n_dev, self.offh_dev, self.hint,
                                    stream, self.scratch)

    def launches(self) -> int:
        """Kernels one run() launches."""
        k = self.batch.count
        pred = (self.ws.weights_launches(k) if self.mode == "guided"
                else self.ws.hint_launches(k))
        return pred + self.db.plan.launches()

    def run(self, stream=None) -> None:
        self.predict(stream)
        if self.mode == "guided":
            self.db.run(stream, weight=self.weight)
        else:
            self.db.run(stream, hint=self.hint)

    def result(self):
        return self.db.result()

    def _learned(self):
        """The C ABI's learned solver (blpg_learned) for this batch's shape."""
        if self._cl is None:
            from .solver import options
            mean = np.ascontiguousarray(self.ws.mean.cpu().numpy(), dtype=np.float32)
            std = np.ascontiguousarray(self.ws.std.cpu().numpy(), dtype=np.float32)
            o = options(self.precision, **self.opts)
            bst = self.batch.c_struct()
            h = C.c_void_p()
            N.check(N.lib().blpg_learned_create(
                self.ws.mlp.h, self.ws.F, mean.ctypes.data_as(C.POINTER(C.c_float)),
                std.ctypes.data_as(C.POINTER(C.c_float)), float(self.beta), C.byref(bst),
                C.byref(o), C.byref(h)), "blpg_learned_create")
            self._cl = h
        return self._cl

    def close(self):
        if self._cl is not None:
            N.lib().blpg_learned_destroy(self._cl)
            self._cl = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, batch: LPBatch, want_x: bool = False):
        """End to end from host arrays (same shapes and offsets as at
        construction): upload A, b, c, predict, solve, download results.
        Guided mode: one call of blpg_learned_solve (the C ABI)."""
        if self.mode == "guided":
            from .solver import SolveResult
            h = self._learned()
            k = batch.count
            st = np.zeros(k, np.int32)
            ob = np.zeros(k, np.float64)
            pv = np.zeros(k, np.int32)
            info = np.zeros(k, np.int32)
            x = None
            if want_x:
                _, _, oc = batch.offsets()
                x = np.zeros(int((oc + batch.n).max()))
            res = N.Result(N.ptr(st, C.c_int32), N.ptr(ob, C.c_double), N.ptr(x, C.c_double),
                           N.ptr(pv, C.c_int32), None, N.ptr(info, C.c_int32))
            fam = np.ascontiguousarray(batch.family, dtype=np.int32)
            bst = batch.c_struct()
            N.check(N.lib().blpg_learned_solve(h, C.byref(bst), N.ptr(fam, C.c_int32),
                                               C.byref(res)), "blpg_learned_solve")
            return SolveResult(st, ob, pv, x, None, info)
        torch = self.torch
        # asynchronous when the host arrays are pinned (stream-ordered before
        # the solve; result() synchronises)
        self.db.A.copy_(torch.from_numpy(batch.A), non_blocking=True)
        self.db.b.copy_(torch.from_numpy(batch.b), non_blocking=True)
        self.db.c.copy_(torch.from_numpy(batch.c), non_blocking=True)
        self.d["fam"].copy_(torch.from_numpy(batch.family.astype(np.int32)))
        self.run()
        return self.db.result()
