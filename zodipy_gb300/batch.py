"""Many observers / epochs with uneven pixel counts in one launch.

The reference evaluates one instant per call (``zodipy/model.py:205-279``) and
spreads a call's pixels over a fork pool (``model.py:182-200``).  Here all
observers' pixels are flattened into one (3, N_total) array; an observer
table with a prefix sum of the pixel counts (``ZlObserver.pix_begin``) lets
every thread find its observer by binary search, so one grid-stride launch
sized to the GPU (SMs x blocks per SM) integrates every line of sight of
every observer, however uneven the counts.  The launch is recorded once into
a CUDA graph and replayed; its shape (threads per block, blocks per SM) comes
from a small autotuner whose choices are cached per GPU and workload.

Each observer keeps the reference's per-call semantics for the cutoff rule
(``zodipy/line_of_sight.py:72-73``): the flags are computed per observer.
"""

from __future__ import annotations

import json
import os

import numpy as np
import torch

from . import _lib, engine, packing

TPB_CHOICES = (32, 64, 96, 128)
BPS_CHOICES = (0, 1, 2, 3, 4, 6, 8, 12, 16, 32, 64)  # 0: the library default, one pixel per thread
CACHE_PATH = os.environ.get("ZODIGB_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "zodigb_tune.json"))


class BatchEvaluator:
    """One model, many observers, one launch.

    ``obs_pos``: (3, n_obs) AU; ``counts``: pixels per observer (sum N);
    ``earth_pos``: (3,) or (3, n_obs).  ``unit_vectors``: (3, N) float64 on
    the device (observer-major: the first counts[0] pixels belong to observer
    0, ...).  Outputs are preallocated: ``total`` (n_spec, N) and optionally
    ``comps`` (n_spec, C, N).
    """

    def __init__(self, zl_model, unit_vectors, obs_pos, counts, earth_pos, precision="float32", comps=False):
        self.zl = _lib.ZlModel.from_buffer_copy(zl_model)
        self.u = unit_vectors
        if not (isinstance(self.u, torch.Tensor) and self.u.is_cuda and self.u.dtype == torch.float64):
            raise ValueError("unit_vectors must be a float64 CUDA tensor (3, N)")
        counts = np.asarray(counts, dtype=np.int64)
        self.n = int(self.u.shape[1])
        if counts.sum() != self.n:
            raise ValueError(f"counts sum to {counts.sum()}, unit_vectors have {self.n} pixels")
        obs = np.asarray(obs_pos, dtype=np.float64).reshape(3, -1)
        if obs.shape[1] != counts.size:
            raise ValueError("one observer position per count")
        begin = np.concatenate([[0], np.cumsum(counts)[:-1]])
        table = packing.observer_table(self.zl, obs, earth_pos, begin, any_mode=False)
        self.obs_dev = engine.upload_observers(table, self.u.device)
        self.n_obs = counts.size
        self.prec = engine.precision_code(precision)
        ns, nc = self.zl.n_spec, self.zl.n_comps
        self.total = torch.empty((ns, self.n), dtype=torch.float64, device=self.u.device)
        self.comps = torch.empty((ns, nc, self.n), dtype=torch.float64, device=self.u.device) if comps else None
        self.graph = None
        self.launch = (0, 0)

    # -- execution -----------------------------------------------------------
    def run(self, stream=None):
        engine.forward(
            self.zl,
            self.u,
            self.obs_dev,
            self.n_obs,
            self.prec,
            want_comps=self.comps is not None,
            want_total=True,
            out_comps=self.comps,
            out_total=self.total,
            stream=stream,
        )
        return self.total

    def set_launch(self, tpb: int, bps: int) -> None:
        _lib.check(_lib.load().zl_set_launch(self.prec, tpb, bps), "zl_set_launch")
        self.launch = (tpb, bps)

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
        return (f"v2|{props.name}|sm{props.multi_processor_count}|p{self.prec}|c{comp}|s{self.zl.n_spec}"
                f"|k{self.zl.n_nodes}")

    def autotune(self, sample: int | None = 1 << 21, reps: int = 3, use_cache: bool = True):
        """Time every (threads per block, blocks per SM) on a sample; keep the fastest.

        The sample is the first ``sample`` pixels (all observers' geometry is
        alike, so per-pixel cost is uniform).  Results are cached per GPU and
        workload signature.  Returns (tpb, bps, ms_per_launch_on_sample).
        """
        key = self._key()
        cache = _load_cache() if use_cache else {}
        if key in cache:
            tpb, bps, ms = cache[key]
            self.set_launch(tpb, bps)
            return tpb, bps, ms
        n = self.n if sample is None else min(self.n, int(sample))
        u = self.u[:, :n]
        out = torch.empty((self.zl.n_spec, n), dtype=torch.float64, device=self.u.device)
        best = None
        for tpb in TPB_CHOICES:
            for bps in BPS_CHOICES:
                self.set_launch(tpb, bps)
                engine.forward(self.zl, u, self.obs_dev, self.n_obs, self.prec, want_comps=False, out_total=out)
                torch.cuda.synchronize()
                ts = []
                for _ in range(reps):
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record()
                    engine.forward(self.zl, u, self.obs_dev, self.n_obs, self.prec, want_comps=False, out_total=out)
                    b.record()
                    ts.append((a, b))
                torch.cuda.synchronize()
                ms = min(a.elapsed_time(b) for a, b in ts)
                if best is None or ms < best[2]:
                    best = (tpb, bps, ms)
        self.set_launch(best[0], best[1])
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
