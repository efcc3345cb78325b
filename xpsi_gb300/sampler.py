"""Sampler-side batching: a vectorised likelihood for samplers that propose
many points at once.

X-PSI's sampler wrappers evaluate one point per likelihood call
(xpsi/UltranestSampler.py:79-96 calls Likelihood.__call__ per point;
xpsi/Sample.py:32-102 runs one MPI rank per point).  BatchedLikelihood takes
a sampler's [n, d] points in the sampler's own parameter order and returns
[n] log-likelihoods from batched GPU evaluations (up to `max_batch` points
per launch), so that

    ultranest.ReactiveNestedSampler(names, BatchedLikelihood(model, names),
                                    transform, vectorized=True)
    emcee.EnsembleSampler(nwalkers, d, BatchedLikelihood(model, names),
                          vectorize=True)

evaluate a whole batch of proposals per call.  Points whose evaluation ends
in one of the reference's early exits get a value near llzero
(Likelihood.random_near_llzero), or -inf with `exit_value="-inf"`."""
from typing import Dict, Optional, Sequence

import numpy as np

from . import batch as BT


def column_map(model: BT.Model, names: Optional[Sequence[str]],
               fixed: Optional[Dict[str, float]]):
    """For each parameter of the model (batch.param_names order), the column
    of the sampler's points that holds it, or None when it is fixed."""
    ours = BT.param_names(model)
    fixed = dict(fixed or {})
    if names is None:
        names = [n for n in ours if n not in fixed]
    names = list(names)
    unknown = [n for n in names if n not in ours]
    if unknown:
        raise KeyError("parameters not in the model: %s" % unknown)
    cols = []
    for n in ours:
        if n in names:
            cols.append(names.index(n))
        elif n in fixed:
            cols.append(None)
        else:
            raise KeyError("parameter %r is neither sampled nor fixed" % n)
    return ours, names, cols, fixed


class BatchedLikelihood:
    """Vectorised log-likelihood over a sampler's [n, d] points.

    names: the sampler's parameter names in column order (default: the
    model's parameters that are not fixed, in batch.param_names order).
    fixed: values of model parameters the sampler does not vary."""

    def __init__(self, model: BT.Model, names: Optional[Sequence[str]] = None,
                 fixed: Optional[Dict[str, float]] = None, precision: str = "plain",
                 device: int = 0, max_batch: int = 4096, exit_value: str = "llzero",
                 evaluator=None):
        if exit_value not in ("llzero", "-inf"):
            raise ValueError("exit_value must be 'llzero' or '-inf'")
        self.model = model
        self.ours, self.names, self.cols, self.fixed = column_map(model, names, fixed)
        self.max_batch = int(max_batch)
        self.exit_value = exit_value
        self.ev = evaluator if evaluator is not None else \
            BT.BatchEvaluator(model, device=device, precision=precision)
        self.calls = 0
        self.points = 0

    @property
    def ndim(self):
        return len(self.names)

    def full_vectors(self, points: np.ndarray) -> np.ndarray:
        """The model's parameter vectors [n, P] from the sampler's points."""
        pts = np.atleast_2d(np.asarray(points, dtype=np.float64))
        if pts.shape[1] != len(self.names):
            raise ValueError("expected %d columns (%s)" % (len(self.names), self.names))
        out = np.empty((pts.shape[0], len(self.ours)))
        for j, (n, c) in enumerate(zip(self.ours, self.cols)):
            out[:, j] = self.fixed[n] if c is None else pts[:, c]
        return out

    def __call__(self, points) -> np.ndarray:
        full = self.full_vectors(points)
        ll = np.empty(full.shape[0])
        starts = list(range(0, full.shape[0], self.max_batch))
        chunks = [full[s:s + self.max_batch] for s in starts]
        if len(chunks) > 1 and hasattr(self.ev, "loglikelihood_pipelined"):
            # several batches: two in flight on separate streams
            results = self.ev.loglikelihood_pipelined(chunks)
        else:
            results = (self.ev.loglikelihood(c) for c in chunks)
        for s, (part, st) in zip(starts, results):
            if self.exit_value == "-inf":
                part = np.where(st != 0, -np.inf, part)
            ll[s:s + self.max_batch] = part
        self.calls += 1
        self.points += full.shape[0]
        return ll
