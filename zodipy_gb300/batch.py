"""Many observers / epochs with uneven pixel counts in one launch.

The reference evaluates one instant per call (``zodipy/model.py:205-279``) and
spreads a call's pixels over a fork pool (``model.py:182-200``).  Here all
observers' pixels are flattened into one (3, N_total) array; an observer
table with a prefix sum of the pixel counts (``ZlObserver.pix_begin``) lets
every thread find its observer by binary search, so one launch integrates
every line of sight of every observer, however uneven the counts.

The launch is persistent: its blocks pull tiles of pixels from a device work
queue (``ZlLaunch.tile``) until the batch is done, so blocks that draw cheap
tiles take more of them; the queue resets itself at the end of the launch,
and the launch is recorded once into a CUDA graph and replayed.  Before that,
each observer's directions are sorted by ecliptic latitude (once, when the
batch is built), so that a warp's lines of sight are alike and the kernels can
skip the dust bands' zero tails for the whole warp; the kernel writes every
result to its caller's column (``ZlLaunch.out_index``), so the outputs keep
the input order.  A small autotuner written for this library picks the block
shape, the tile size and the number of resident blocks per SM by timing the
candidates on a sample of the batch; its choices are cached per GPU and
workload and held by the evaluator (no process-wide launch state).

Each observer keeps the reference's per-call semantics for the cutoff rule
(``zodipy/line_of_sight.py:72-73``): the flags are computed per observer.
"""

from __future__ import annotations

import json
import os

import numpy as np
import torch

from . import _lib, engine, packing

# (threads per block, blocks per SM, tile in items, band tails); blocks per SM 0 with tile 0 = the
# static one-block-per-tile launch.  Band tails (skipping the dust bands' zero terms for a whole
# warp) pay only where a warp's lines of sight are alike, and cost a test per node where they are
# not, so the tuner times both on a sorted batch.
STATIC_CHOICES = tuple((tpb, 0, 0, tails) for tpb in (64, 96, 128) for tails in (False, True))
QUEUE_CHOICES = tuple((tpb, bps, tpb * k, tails) for tpb in (64, 128) for bps in (2, 4, 6, 8, 16) for k in (1, 2, 4, 8)
                      for tails in (False, True))
CACHE_PATH = os.environ.get("ZODIGB_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "zodigb_tune.json"))


class BatchEvaluator:
    """One model, many observers, one launch.

    ``obs_pos``: (3, n_obs) AU; ``counts``: pixels per observer (sum N);
    ``earth_pos``: (3,) or (3, n_obs).  ``unit_vectors``: (3, N) float64 on
    the device (observer-major: the first counts[0] pixels belong to observer
    0, ...).  Outputs are preallocated, in the input order: ``total``
    (n_spec, N) and optionally ``comps`` (n_spec, C, N).  ``sort`` (default)
    evaluates each observer's directions in order of latitude (a sorted copy of
    the unit vectors is kept; results are the same bits either way).
    """

    def __init__(self, zl_model, unit_vectors, obs_pos, counts, earth_pos, precision="float32", comps=False,
                 sort=True):
        self.zl = _lib.ZlModel.from_buffer_copy(zl_model)
        u = unit_vectors
        if not (isinstance(u, torch.Tensor) and u.is_cuda and u.dtype == torch.float64):
            raise ValueError("unit_vectors must be a float64 CUDA tensor (3, N)")
        counts = np.asarray(counts, dtype=np.int64)
        self.n = int(u.shape[1])
        if counts.sum() != self.n:
            raise ValueError(f"counts sum to {counts.sum()}, unit_vectors have {self.n} pixels")
        obs = np.asarray(obs_pos, dtype=np.float64).reshape(3, -1)
        if obs.shape[1] != counts.size:
            raise ValueError("one observer position per count")
        dev = u.device
        begin = np.concatenate([[0], np.cumsum(counts)[:-1]])
        table = packing.observer_table(self.zl, obs, earth_pos, begin, any_mode=False)
        self.obs_dev = engine.upload_observers(table, dev)
        self.n_obs = counts.size
        self.prec = engine.precision_code(precision)
        self.sorted = bool(sort)
        if self.sorted:
            # observer index + (sin(latitude) + 1) in [0, 2): one stable sort orders every
            # observer's pixels by latitude and keeps the observers in place
            owner = torch.repeat_interleave(torch.arange(self.n_obs, device=dev, dtype=torch.float64),
                                            torch.from_numpy(counts).to(dev))
            self.order = torch.sort(owner * 4.0 + (u[2] + 1.0), stable=True).indices
            del owner
            self.u = u[:, self.order].contiguous()
        else:
            self.order = None
            self.u = u.contiguous()
        ns, nc = self.zl.n_spec, self.zl.n_comps
        self.total = torch.empty((ns, self.n), dtype=torch.float64, device=dev)
        self.comps = torch.empty((ns, nc, self.n), dtype=torch.float64, device=dev) if comps else None
        self.queue = torch.zeros(2, dtype=torch.int32, device=dev)
        self.graph = None
        self.set_launch(128, 8, 256, False)

    # -- execution -----------------------------------------------------------
    def _options(self, tpb: int, bps: int, tile: int, tails: bool) -> _lib.ZlLaunch:
        return engine.launch_options(threads_per_block=tpb, blocks_per_sm=bps, band_tails=tails, tile=tile,
                                     queue=self.queue if tile > 0 else None, out_index=self.order)

    def run(self, stream=None, n: int | None = None):
        """One launch over the batch (the first ``n`` pixels of its evaluation order if given)."""
        u = self.u if n is None else self.u[:, :n]
        engine.forward(
            self.zl,
            u,
            self.obs_dev,
            self.n_obs,
            self.prec,
            want_comps=self.comps is not None and n is None,
            want_total=True,
            out_comps=self.comps if n is None else None,
            out_total=self.total,
            stream=stream,
            launch=self.launch_opt,
        )
        return self.total

    def set_launch(self, tpb: int, bps: int, tile: int = 0, tails: bool = False) -> None:
        """This evaluator's launch shape (other evaluators and models are not affected)."""
        self.launch = (int(tpb), int(bps), int(tile), bool(tails))
        self.launch_opt = self._options(*self.launch)
        self.graph = None

    def capture(self):
        """Record one launch into a CUDA graph (call after tuning)."""
        s = torch.cuda.Stream(self.u.device)
        s.wait_stream(torch.cuda.current_stream(self.u.device))
        with torch.cuda.stream(s):
            self.run()  # warm-up outside the graph
        torch.cuda.current_stream(self.u.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return self.total

    # -- autotuning ------------------------------------------------------------
    def _key(self) -> str:
        props = torch.cuda.get_device_properties(self.u.device)
        comp = "".join(str(self.zl.comp[c].type) for c in range(self.zl.n_comps))
        return (f"v4|{props.name}|sm{props.multi_processor_count}|p{self.prec}|c{comp}|s{self.zl.n_spec}"
                f"|k{self.zl.n_nodes}|sorted{int(self.sorted)}")

    def autotune(self, sample: int | None = 1 << 21, reps: int = 3, use_cache: bool = True):
        """Time every candidate (threads per block, blocks per SM, tile, band tails) on a sample;
        keep the fastest.

        Candidates: the static one-block-per-tile launch and work-queue launches of several
        tile sizes and grid caps, each with and without band tails (without only, for an
        unsorted batch, whose warps are too mixed for them).  The sample is the first ``sample`` pixels of the evaluation
        order (whole observers, whose directions span every latitude).  Results are cached per
        GPU and workload signature.  Returns (tpb, bps, tile, tails, ms_per_launch_on_sample).
        """
        key = self._key()
        cache = _load_cache() if use_cache else {}
        if key in cache:
            tpb, bps, tile, tails, ms = cache[key]
            self.set_launch(tpb, bps, tile, tails)
            return tpb, bps, tile, bool(tails), ms
        n = self.n if sample is None else min(self.n, int(sample))
        best = None
        for cand in STATIC_CHOICES + QUEUE_CHOICES:
            if cand[3] and not self.sorted:
                continue
            self.set_launch(*cand)
            self.run(n=n)
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                self.run(n=n)
                b.record()
                ts.append((a, b))
            torch.cuda.synchronize()
            ms = min(a.elapsed_time(b) for a, b in ts)
            if best is None or ms < best[4]:
                best = (*cand, ms)
        self.set_launch(*best[:4])
        if use_cache:
            cache[key] = list(best)
            _save_cache(cache)
        return best


def _load_cache() -> dict:
    try:
        with open(CACHE_PATH) as f:
            return json.load(f)
    except Exception:
        return {}


def _save_cache(cache: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        tmp = CACHE_PATH + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, CACHE_PATH)
    except OSError:
        pass


def uneven_observers(n_obs: int, seed: int, lo: int = 10_000, hi: int = 500_000):
    """Observers on a 1 AU circle (angle U(0, 2pi), z ~ N(0, 0.01) AU) with pixel counts U{lo..hi}."""
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0.0, 2 * np.pi, n_obs)
    z = rng.normal(0.0, 0.01, n_obs)
    obs = np.stack([np.cos(phi), np.sin(phi), z])
    counts = rng.integers(lo, hi + 1, n_obs)
    return obs, counts


def random_directions_device(n: int, seed: int, device="cuda") -> torch.Tensor:
    """(3, n) float64 unit vectors uniform on the sphere (normalised Gaussians), generated on the device."""
    g = torch.Generator(device).manual_seed(seed)
    v = torch.randn((3, n), dtype=torch.float64, device=device, generator=g)
    return v / v.norm(dim=0, keepdim=True)
