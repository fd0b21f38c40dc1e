"""Many independent GP + MC-acquisition problems in one CUDA-graph launch.

Each problem keeps its own model, acquisition object, candidate shape and
buffers. ``ModelBatch`` captures every problem's value + gradient call into
one CUDA graph spread over several streams (longest problems first onto the
least-loaded stream), so that evaluating all problems is one graph launch from
the host and small problems run side by side on the GPU. ``Autotuner`` picks,
per (n bucket, d, b, q, precision) bucket, the schedule of a problem -- the
cross-covariance GEMM form (tcgen05 tensor cores or FFMA, mixed path) and the
adjoint contraction's CTA target -- by timing the candidates on the bucket's
first problem and reusing the winner for the rest of the bucket.

The many-model configuration of the reference's optimisation loop evaluates
each model's acquisition separately (botorch/generation/gen.py:423-487, one
model per ``optimize_acqf`` call); this module batches those evaluations.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import torch
from torch import Tensor

from botorch_gb300 import _native as nat
from botorch_gb300.exceptions import UnsupportedError

# (tensor-core GEMMs, adjoint CTAs per SM); 0 = the library default
SCHEDULES: tuple[tuple[bool, int], ...] = ((True, 0), (True, 8), (True, 32), (False, 0), (False, 8))


def bucket_key(n: int, d: int) -> tuple[int, int]:
    """Problems share a schedule bucket when their n rounds up to the same power of two
    and their d is equal."""
    return (1 << max(0, int(n - 1).bit_length()), int(d))


def assign_streams(costs: list[float], n_streams: int) -> list[list[int]]:
    """Longest-first list scheduling: each problem (in decreasing cost) goes to the
    stream with the least total cost so far. Returns the problem indices per stream."""
    if n_streams < 1:
        raise ValueError("n_streams must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * n_streams
    lanes: list[list[int]] = [[] for _ in range(n_streams)]
    for i in order:
        k = min(range(n_streams), key=lambda j: (loads[j], j))
        lanes[k].append(i)
        loads[k] += costs[i]
    return lanes


def apply_schedule(acqf, schedule: tuple[bool, int]) -> None:
    acqf.use_tensor_cores = bool(schedule[0])
    acqf.adjoint_ctas_per_sm = int(schedule[1])


def time_call(acqf, Xd: Tensor, out, ws, repeats: int = 3) -> float:
    """Mean device time (ms) of one value + gradient call, after one warm-up call."""
    stream = torch.cuda.current_stream(Xd.device)
    acqf.value_and_grad_raw(Xd, True, check=False, out=out, ws=ws)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(repeats):
        acqf.value_and_grad_raw(Xd, True, check=False, out=out, ws=ws)
    stop.record(stream)
    stop.synchronize()
    return start.elapsed_time(stop) / repeats


@dataclass
class Autotuner:
    """Per-bucket schedule choice by timing; ``choice`` and ``timings`` are kept for reports."""

    schedules: tuple[tuple[bool, int], ...] = SCHEDULES
    repeats: int = 3
    choice: dict = field(default_factory=dict)
    timings: dict = field(default_factory=dict)

    def key(self, acqf, Xd: Tensor) -> tuple:
        return bucket_key(acqf.model.n, acqf.model.d) + (int(Xd.shape[0]), int(Xd.shape[1]),
                                                          acqf.precision)

    def tune(self, acqf, Xd: Tensor, out, ws) -> tuple[bool, int]:
        key = self.key(acqf, Xd)
        if key not in self.choice:
            cands = [s for s in self.schedules if acqf.precision == "mixed" or not s[0]]
            if not cands:
                cands = [(False, 0)]
            times = {}
            for sched in cands:
                apply_schedule(acqf, sched)
                times[sched] = time_call(acqf, Xd, out, ws, self.repeats)
            self.timings[key] = times
            self.choice[key] = min(times, key=times.get)
        apply_schedule(acqf, self.choice[key])
        return self.choice[key]


class ModelBatch:
    """Value + gradient of many acquisition problems per graph launch.

    ``acqfs[i]`` evaluates candidates of shape ``shapes[i] = (b_i, q_i, d_i)``
    (float64, on the acquisitions' device). ``value_and_grad(Xs)`` copies the
    candidates into the captured inputs, replays the graph and returns
    ``[(value_i, grad_i)]``, views of the graph's output buffers that the next
    call overwrites.
    """

    def __init__(self, acqfs: list, shapes: list[tuple[int, int, int]], n_streams: int = 4,
                 tuner: Autotuner | None = None) -> None:
        if len(acqfs) != len(shapes) or not acqfs:
            raise ValueError("one candidate shape per acquisition function is required")
        self.acqfs = acqfs
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        self.device = acqfs[0].device
        self.n_streams = max(1, min(int(n_streams), len(acqfs)))
        self.tuner = tuner
        self.graph = None
        self.launches = 0
        self.costs: list[float] = []
        self.lanes: list[list[int]] = []

    def _capture(self, Xs: list[Tensor]) -> None:
        dev = self.device
        self.X = [x.detach().to(dev, torch.float64).contiguous().clone() for x in Xs]
        self.out = [(torch.empty(b, dtype=torch.float64, device=dev),
                     torch.empty(b, q, d, dtype=torch.float64, device=dev),
                     torch.empty(b, dtype=torch.int32, device=dev)) for b, q, d in self.shapes]
        self.ws = [nat.Workspace(dev) for _ in self.acqfs]
        self.costs = []
        for i, a in enumerate(self.acqfs):
            if self.tuner is not None:
                self.tuner.tune(a, self.X[i], self.out[i], self.ws[i])
            self.costs.append(time_call(a, self.X[i], self.out[i], self.ws[i], 1))
        self.lanes = assign_streams(self.costs, self.n_streams)
        streams = [torch.cuda.Stream(dev) for _ in range(self.n_streams)]
        torch.cuda.synchronize(dev)
        lib = nat.lib()
        graph = torch.cuda.CUDAGraph()
        n0 = lib.bgb_launch_count()
        with torch.cuda.graph(graph):
            main = torch.cuda.current_stream(dev)
            for s in streams:
                s.wait_stream(main)
            for s, lane in zip(streams, self.lanes):
                with torch.cuda.stream(s):
                    for i in lane:
                        self.acqfs[i].value_and_grad_raw(self.X[i], True, check=False,
                                                         out=self.out[i], ws=self.ws[i])
            for s in streams:
                main.wait_stream(s)
        self.launches = lib.bgb_launch_count() - n0
        self.graph = graph
        # the call structs (and the base samples they point to) the graph was captured with
        self.structs = [a._call_struct(s[1])[0] for a, s in zip(self.acqfs, self.shapes)]
        self.keep = [a._Z.get(s[1]) for a, s in zip(self.acqfs, self.shapes)]

    def _stale(self) -> bool:
        """A problem's call struct changed (new baseline or pending points): its graph
        would read released buffers, so it has to be captured again."""
        return any(a._call_struct(s[1])[0] is not st
                   for a, s, st in zip(self.acqfs, self.shapes, self.structs))

    def value_and_grad(self, Xs: list[Tensor], check: bool = True) -> list[tuple[Tensor, Tensor]]:
        if len(Xs) != len(self.acqfs):
            raise ValueError("one candidate tensor per acquisition function is required")
        for x, s in zip(Xs, self.shapes):
            if tuple(x.shape) != s:
                raise ValueError(f"candidate shape {tuple(x.shape)} differs from the captured {s}")
        if self.graph is None or self._stale():
            self._capture(Xs)
        else:
            for dst, x in zip(self.X, Xs):
                dst.copy_(x)
        self.graph.replay()
        if check:
            worst = int(torch.stack([o[2].max() for o in self.out]).max().item())
            if worst != 0:
                self.acqfs[0]._raise_for_status(torch.tensor([worst]))
        return [(o[0], o[1]) for o in self.out]


class ModelGroup:
    """Value + gradient of many acquisition problems with one launch per stage.

    A native group plan (``bgb_group_*``) runs every problem's kernel build,
    forward tensor-core GEMM, covariance reduction, batch step, row mix, adjoint
    GEMM and adjoint as one launch each over all problems (about ten kernels
    for the whole group, captured in one CUDA graph), instead of ~11 launches
    per problem. Members must be mixed-precision tensor-core problems with a
    cached root, q <= 8 and r <= 4; ``ModelGroup.supported`` says whether a set
    qualifies. ``value_and_grad(Xs)`` copies the candidates into the plan's
    inputs, replays the graph and returns ``[(value_i, grad_i)]`` (views that the
    next call overwrites). With ``check`` (default), a problem whose status
    reports a failed low-rank update is evaluated again on its own, through its
    acquisition function's fallback to joint sampling.
    """

    def __init__(self, acqfs: list, shapes: list[tuple[int, int, int]]) -> None:
        if len(acqfs) != len(shapes) or not acqfs:
            raise ValueError("one candidate shape per acquisition function is required")
        self.acqfs = acqfs
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        self.device = acqfs[0].device
        self.handle = None
        self.graph = None
        self.launches = 0
        self._build()

    @staticmethod
    def _structs(acqfs, shapes):
        return [a._call_struct(s[1])[0] for a, s in zip(acqfs, shapes)]

    @classmethod
    def supported(cls, acqfs: list, shapes: list[tuple[int, int, int]]) -> bool:
        structs = cls._structs(acqfs, shapes)
        arr = (nat.BgbAcq * len(structs))(*structs)
        b = (ctypes.c_int64 * len(shapes))(*[int(s[0]) for s in shapes])
        return nat.lib().bgb_group_workspace_bytes(arr, b, len(structs)) > 0

    def _build(self) -> None:
        dev, lib = self.device, nat.lib()
        self.close()
        self.structs = self._structs(self.acqfs, self.shapes)
        count = len(self.structs)
        self._arr = (nat.BgbAcq * count)(*self.structs)
        self._b = (ctypes.c_int64 * count)(*[s[0] for s in self.shapes])
        wsb = lib.bgb_group_workspace_bytes(self._arr, self._b, count)
        if wsb == 0:
            raise UnsupportedError("ModelGroup members must be mixed-precision tensor-core problems "
                                   "with a cached root, q <= 8 and r <= 4")
        self.X = [torch.zeros(s, dtype=torch.float64, device=dev) for s in self.shapes]
        self.out = [(torch.empty(b, dtype=torch.float64, device=dev),
                     torch.empty(b, q, d, dtype=torch.float64, device=dev),
                     torch.empty(b, dtype=torch.int32, device=dev)) for b, q, d in self.shapes]
        self.ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        ptrs = lambda ts: (ctypes.c_void_p * count)(*[t.data_ptr() for t in ts])  # noqa: E731
        handle = ctypes.c_void_p()
        with torch.cuda.device(dev):
            rc = lib.bgb_group_create(self._arr, self._b, count, ptrs(self.X),
                                      ptrs([o[0] for o in self.out]), ptrs([o[1] for o in self.out]),
                                      ptrs([o[2] for o in self.out]), self.ws.data_ptr(), wsb,
                                      nat.stream_handle(dev), ctypes.byref(handle))
        nat.check(rc, "model group plan")
        self.handle = handle
        self.launches = int(lib.bgb_group_launches(handle))
        # the base samples the structs point to stay alive with the plan
        self._keep = [a._Z.get(s[1]) for a, s in zip(self.acqfs, self.shapes)]
        torch.cuda.synchronize(dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            nat.check(lib.bgb_group_run(self.handle, nat.stream_handle(dev)), "model group run")
        self.graph = graph

    def _stale(self) -> bool:
        return any(a._call_struct(s[1])[0] is not st
                   for a, s, st in zip(self.acqfs, self.shapes, self.structs))

    def value_and_grad(self, Xs: list[Tensor], check: bool = True) -> list[tuple[Tensor, Tensor]]:
        if len(Xs) != len(self.acqfs):
            raise ValueError("one candidate tensor per acquisition function is required")
        for x, s in zip(Xs, self.shapes):
            if tuple(x.shape) != s:
                raise ValueError(f"candidate shape {tuple(x.shape)} differs from the plan's {s}")
        if self._stale():
            self._build()
        for dst, x in zip(self.X, Xs):
            dst.copy_(x)
        self.graph.replay()
        res = [(o[0], o[1]) for o in self.out]
        if check:
            bad = [i for i, o in enumerate(self.out) if int(o[2].max().item()) != 0]
            for i in bad:  # the problem's own path: fallback to joint sampling, or the error
                res[i] = self.acqfs[i].value_and_grad_raw(self.X[i], True)
        return res

    def close(self) -> None:
        if self.handle is not None:
            if self.graph is not None:
                torch.cuda.synchronize(self.device)
            nat.lib().bgb_group_destroy(self.handle)
            self.handle = None
            self.graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover - interpreter shutdown
            pass
