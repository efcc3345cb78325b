"""A request loop on one GPU for sampler likelihood calls (continuous batching).

Requests -- (model name, parameter vectors [V, P]) with V from 1 to thousands --
arrive at any time through submit(); each returns a Future of
(log L [V], status [V]).  Models (shape classes: hot-region kinds, mesh
resolutions, leaves, rays, energies) are registered once and their atmosphere
table, response matrix, data and grids stay resident on the device.

Pipeline:
  submit -> host preparation thread(s): derived quantities and cell budgets
            (the meshes themselves are built on the GPU at admission, or on
            the host with meshes="host")
         -> ready queue
         -> dispatcher: requests of one model that are ready together are
            merged into one launch (up to max_vectors); a launch is admitted
            when one of `slots` CUDA streams is free AND its estimated device
            footprint fits the HBM budget left; admitted launches run
            concurrently on their streams
         -> completion polling (CUDA events): results copied back, futures
            resolved, memory and slot released.

A request that arrives while others run is admitted as soon as a slot and
memory free up, and its kernels overlap with theirs on the device.
Latencies (arrival to result) are recorded per request.
"""
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import batch as BT


@dataclass(eq=False)
class _Req:
    model: str
    params: np.ndarray
    future: Future
    t_submit: float
    prepared: object = None
    t_ready: float = 0.0


@dataclass(eq=False)
class _Launch:
    model: str
    reqs: list
    slot: int
    B: dict
    event: object
    nbytes: int
    t_start: float


@dataclass
class ServerStats:
    latencies: list = field(default_factory=list)
    vectors: int = 0
    launches: int = 0
    merged_requests: int = 0
    peak_concurrency: int = 0
    peak_bytes: int = 0


def estimate_bytes(ev: BT.BatchEvaluator, P) -> int:
    """Device footprint of one prepared launch (inputs, ray tables, fluxes,
    integrated signals, folded signals, likelihood scratch, integrator
    partials and table slabs)."""
    n_m = P.V * P.H
    N_E = len(ev.model.energies)
    N_P = ev.N_L
    # packed rows (8 FP64 + mesh index) and cells (area, azimuth, 2 params,
    # flag), whether uploaded or built on the device, plus the GPU mesh
    # builder's scratch (area tables, per-row temporaries)
    b = P.n_rows * (8 * 8 + 4) + P.n_cells * (4 * 8 + 4) + P.d_sq.nbytes + P.shifts.nbytes
    b += len(P.meshes) * 1000 * 8 + P.n_rows * 4 * 8
    b += 3 * P.n_rows * ev.N_R * 8 + P.n_rows * 12
    b += n_m * (N_E * N_P + ev.q * N_P + ev.K * N_P) * 8
    b += P.V * ev.K * 12 + P.V * 12
    b += 8 * 152 * (N_E * N_P * 8)           # chunk partials (bounded)
    if ev.atmos is not None:
        b += 8 * 152 * ev.atmos.nmu * ev.atmos.nE * 8
    if getattr(P, "else_V", 0):
        # elsewhere: packed parallels and cells, ray tables, per-parallel
        # spectra, the spectra, and the hot regions' correction vectors
        er = P.else_V * P.else_S
        b += er * (6 * 8 + 4) + er * P.else_S * 3 * 8
        b += 3 * er * ev.model.elsewhere.num_rays * 8 + er * 12
        b += er * N_E * 8 + P.else_V * (N_E * 8 + 4)
        b += P.n_cells * 2 * 8
    return int(b)


class Server:
    def __init__(self, models: dict, device=0, hbm_budget=120 << 30, slots=4,
                 max_vectors=4096, precision="plain", prep_threads=2, mesh_threads=0,
                 meshes="gpu"):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        self.evals = {name: BT.BatchEvaluator(m, device=device, precision=precision)
                      for name, m in models.items()}
        self.budget = int(hbm_budget)
        self.max_vectors = int(max_vectors)
        self.mesh_threads = mesh_threads
        self.meshes = meshes
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(slots)]
        self.free_slots = list(range(slots))
        self.in_use = 0
        self.inflight = []
        self.incoming = queue.Queue()
        self.ready = []
        self.ready_lock = threading.Lock()
        self.stats = ServerStats()
        self.failed = None
        self._stop = threading.Event()
        self._prep = [threading.Thread(target=self._prep_loop, daemon=True)
                      for _ in range(prep_threads)]
        self._disp = threading.Thread(target=self._dispatch_loop, daemon=True)
        for t in self._prep:
            t.start()
        self._disp.start()

    # ------------------------------------------------------------------ API
    def submit(self, model: str, params) -> Future:
        if model not in self.evals:
            raise KeyError("unknown model %r" % model)
        if self.failed is not None:
            raise RuntimeError("the serving loop stopped") from self.failed
        f = Future()
        self.incoming.put(_Req(model, np.atleast_2d(np.asarray(params, np.float64)), f,
                               time.perf_counter()))
        return f

    def close(self):
        self._stop.set()
        for _ in self._prep:
            self.incoming.put(None)
        for t in self._prep:
            t.join(timeout=30)
        self._disp.join(timeout=60)

    def latency_percentiles(self):
        lat = np.array(self.stats.latencies)
        if lat.size == 0:
            return None
        return {"p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "requests": int(lat.size)}

    # ------------------------------------------------------------------ threads
    def _prep_loop(self):
        while not self._stop.is_set():
            r = self.incoming.get()
            if r is None:
                return
            try:
                r.prepared = BT.prepare(self.evals[r.model].model, r.params, self.mesh_threads,
                                        meshes=self.meshes)
                r.t_ready = time.perf_counter()
                with self.ready_lock:
                    self.ready.append(r)
            except Exception as e:  # noqa: BLE001 - delivered to the caller
                r.future.set_exception(e)

    def _merge(self, reqs):
        """One packed launch from several prepared requests of one model."""
        return BT.concat_prepared([r.prepared for r in reqs], self.evals[reqs[0].model].model)

    def _dispatch_loop(self):
        try:
            self._dispatch()
        except BaseException as e:  # noqa: BLE001 - delivered to every waiting caller
            self._fail_all(e)

    def _fail_all(self, e):
        pending = [r for L in self.inflight for r in L.reqs]
        with self.ready_lock:
            pending += self.ready
            self.ready = []
        while True:
            try:
                r = self.incoming.get_nowait()
            except queue.Empty:
                break
            if r is not None:
                pending.append(r)
        for r in pending:
            if not r.future.done():
                r.future.set_exception(e)
        self.failed = e

    def _dispatch(self):
        torch = self.torch
        torch.cuda.set_device(self.dev)
        while True:
            progressed = self._poll()
            progressed |= self._admit()
            if self._stop.is_set() and not self.inflight and not self.ready \
                    and self.incoming.empty():
                return
            if not progressed:
                time.sleep(0.0005)

    def _poll(self):
        done = [L for L in self.inflight if L.event.query()]
        for L in done:
            self.inflight.remove(L)
            B = L.B
            ev = self.evals[L.model]
            ll = B["loglike"].cpu().numpy()
            st = ev.statuses(B)
            bad = st != 0
            if bad.any():
                rng = np.random.default_rng(int(L.t_start * 1e6) & 0xffffffff)
                ll = ll.copy()
                ll[bad] = ev.model.llzero * (0.1 + 0.9 * rng.random(int(bad.sum())))
            now = time.perf_counter()
            o = 0
            for r in L.reqs:
                n = r.params.shape[0]
                r.future.set_result((ll[o:o + n].copy(), st[o:o + n].copy()))
                self.stats.latencies.append(now - r.t_submit)
                o += n
            self.stats.vectors += o
            self.in_use -= L.nbytes
            self.free_slots.append(L.slot)
        return bool(done)

    def _admit(self):
        admitted = False
        while self.free_slots:
            with self.ready_lock:
                if not self.ready:
                    break
                # oldest ready request's model; merge its peers that are ready
                model = self.ready[0].model
                group, rest, n = [], [], 0
                for r in self.ready:
                    if r.model == model and n + r.params.shape[0] <= self.max_vectors:
                        group.append(r)
                        n += r.params.shape[0]
                    else:
                        rest.append(r)
            ev = self.evals[model]
            P = self._merge(group)
            need = estimate_bytes(ev, P)
            if self.in_use + need > self.budget and self.inflight:
                break  # wait for memory to free up
            taken = set(id(r) for r in group)
            with self.ready_lock:
                self.ready = [r for r in self.ready if id(r) not in taken]
            slot = self.free_slots.pop(0)
            s = self.streams[slot]
            torch = self.torch
            with torch.cuda.stream(s):
                B = ev.upload(P, pinned=True)
                ev.run(B, stream=s)
                e = torch.cuda.Event()
                e.record(s)
            self.in_use += need
            self.stats.peak_bytes = max(self.stats.peak_bytes, self.in_use)
            self.inflight.append(_Launch(model, group, slot, B, e, need, time.perf_counter()))
            self.stats.launches += 1
            self.stats.merged_requests += len(group) - 1
            self.stats.peak_concurrency = max(self.stats.peak_concurrency, len(self.inflight))
            admitted = True
        return admitted


def poisson_stream(rate_hz, duration_s, max_batch, seed=5, min_batch=1):
    """Arrival times and log-uniform batch sizes of a Poisson request stream."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > duration_s:
            break
        v = int(np.exp(rng.uniform(np.log(min_batch), np.log(max_batch + 1))))
        out.append((t, max(min_batch, min(max_batch, v))))
    return out
