"""Many independent 3-D transforms of uneven sizes as one CUDA-graph launch.

Two forms of the same batch:
  * "streams": every instance's own kernels, forked over `streams` CUDA
    streams inside the graph;
  * "grouped": the instances' calls are recorded into an accfft_gb300.Batch
    and run level by level, one persistent grouped kernel per (pass kind,
    line length) and level, whose CTAs walk the tiles of every instance's
    pass (about 10 levels x a few lengths instead of one launch per pass per
    instance).
tune() times both and keeps the faster.

    bp = BatchPlan([((32, 32, 32), "r2c_c2r"), ((160, 180, 200), "lap_invlap"), ...])
    bp.set_inputs(list_of_tensors)      # or bp.inputs[i].copy_(...)
    bp.tune()                            # optional: per-shape schedule and stream count
    bp.capture()
    bp.run()                             # one graph launch for the whole batch
    bp.outputs[i]

Instance operations:
    "r2c_c2r"     out = c2r(r2c(in))          (unnormalised: N * in)     2 transforms
    "laplace"     out = laplace(in)                                        2 transforms
    "inv_laplace" out = inv_laplace(in)                                    2 transforms
    "lap_invlap"  out = inv_laplace(laplace(in))                           4 transforms

Every instance owns its plan (and so its twiddle tables and spectrum scratch),
so instances can run concurrently: the capture forks the work over
`streams` CUDA streams (largest instances first, greedy balance by grid
size) and joins them before the graph ends.

The autotuner times, per distinct grid, the z+y schedules the library offers
for it (separate z and y passes, the cluster slab kernel or the persistent z+y
kernel where the grid has one; accfft_c_set_zy_schedule) and then the number
of capture streams, and
keeps the fastest; schedules are cached per (dtype, shape) in a JSON file if
`cache` is given.  report() lists the compiled radix plan of every axis.
"""
from __future__ import annotations

import json
import os

import torch

from . import AccfftError, Batch, PlanR2C, lib, line_plan

OPS = {"r2c_c2r": 2, "laplace": 2, "inv_laplace": 2, "lap_invlap": 4}


def radix_plan(length: int, dtype: str) -> dict:
    """The compiled radix plan of a line length: first radix E, threads per
    line P and the stage radices (for reports)."""
    return line_plan(length, dtype)


class _Instance:
    def __init__(self, idx, shape, op, dtype, device, flags=None):
        self.idx, self.shape, self.op = idx, tuple(shape), op
        tdt = getattr(torch, dtype)
        self.inp = torch.empty(self.shape, dtype=tdt, device=device)
        self.out = torch.empty(self.shape, dtype=tdt, device=device)
        n0, n1, n2 = self.shape
        self.spec = torch.empty((n0, n1, n2 // 2 + 1, 2), dtype=tdt, device=device) if op == "r2c_c2r" else None
        self.tmp = torch.empty(self.shape, dtype=tdt, device=device) if op == "lap_invlap" else None
        self.plan = None
        self.dtype = dtype
        self.flags = flags

    def make_plan(self, schedule):
        if self.plan is None:
            self.plan = PlanR2C(self.shape, self.dtype, **({} if self.flags is None else {"flags": self.flags}))
        self.plan.set_zy_schedule({"split": 0, "fused": 1, "persistent": 2}[schedule])

    def enqueue(self, stream):
        p = self.plan
        p.set_stream(stream.cuda_stream, blocking=False)
        if self.op == "r2c_c2r":
            p.r2c(self.inp, self.spec)
            p.c2r(self.spec, self.out)
        elif self.op == "laplace":
            p.laplace(self.out, self.inp)
        elif self.op == "inv_laplace":
            p.inv_laplace(self.out, self.inp)
        else:
            p.laplace(self.tmp, self.inp)
            p.inv_laplace(self.out, self.tmp)


class BatchPlan:
    def __init__(self, specs, dtype="float32", streams=4, cache=None, device="cuda", form="streams", flags=None):
        for shape, op in specs:
            if op not in OPS:
                raise ValueError(f"unknown operation {op!r}")
        lib()
        self.dtype = dtype
        self.streams = streams
        self.cache = cache
        self.schedule = {}
        self.instances = [_Instance(i, s, op, dtype, device, flags) for i, (s, op) in enumerate(specs)]
        for inst in self.instances:
            inst.make_plan("split")
        self.graph = None
        self._side = {}
        self.transforms = sum(OPS[i.op] for i in self.instances)
        self.form = form
        self._batch = None

    @property
    def inputs(self):
        return [i.inp for i in self.instances]

    @property
    def outputs(self):
        return [i.out for i in self.instances]

    def set_inputs(self, tensors):
        for inst, t in zip(self.instances, tensors):
            inst.inp.copy_(t)

    # ------------------------------------------------------------ schedule
    def _assign(self, k):
        """greedy balance of the instances over k streams, largest grids first"""
        order = sorted(self.instances, key=lambda i: -i.shape[0] * i.shape[1] * i.shape[2] * OPS[i.op])
        loads = [0] * k
        lanes = [[] for _ in range(k)]
        for inst in order:
            j = loads.index(min(loads))
            lanes[j].append(inst)
            loads[j] += inst.shape[0] * inst.shape[1] * inst.shape[2] * OPS[inst.op]
        return lanes

    def _enqueue_all(self, main, k):
        lanes = self._assign(k)
        if k not in self._side:
            self._side[k] = [torch.cuda.Stream() for _ in range(k)]
        side = self._side[k]
        start = torch.cuda.Event()
        start.record(main)
        ends = []
        for s, lane in zip(side, lanes):
            s.wait_event(start)
            for inst in lane:
                inst.enqueue(s)
            e = torch.cuda.Event()
            e.record(s)
            ends.append(e)
        for e in ends:
            main.wait_event(e)

    def _time_eager(self, k, reps=3):
        main = torch.cuda.current_stream()
        self._enqueue_all(main, k)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(main)
        for _ in range(reps):
            self._enqueue_all(main, k)
        b.record(main)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    def tune(self, stream_choices=(1, 2, 4, 8)):
        """Pick the z+y schedule per distinct grid, then the stream count."""
        cached = {}
        if self.cache and os.path.exists(self.cache):
            cached = json.load(open(self.cache))
        shapes = sorted({i.shape for i in self.instances})
        for shape in shapes:
            key = f"{self.dtype}:{'x'.join(map(str, shape))}"
            if key in cached:
                self.schedule[shape] = cached[key]
                continue
            probe = _Instance(-1, shape, "r2c_c2r", self.dtype, self.instances[0].inp.device, self.instances[0].flags)
            probe.inp.uniform_(-1, 1)
            best = None
            for sched in ("split", "fused", "persistent"):
                try:
                    probe.make_plan(sched)
                except AccfftError:
                    continue            # no slab kernel for this grid
                main = torch.cuda.current_stream()
                probe.enqueue(main)
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(main)
                for _ in range(5):
                    probe.enqueue(main)
                b.record(main)
                torch.cuda.synchronize()
                t = a.elapsed_time(b)
                if best is None or t < best[0]:
                    best = (t, sched)
            probe.plan.destroy()
            self.schedule[shape] = best[1]
            cached[key] = best[1]
        for inst in self.instances:
            inst.make_plan(self.schedule[inst.shape])
        times = {k: self._time_eager(k) for k in stream_choices}
        self.streams = min(times, key=times.get)
        grouped_ms = None
        try:
            grouped_ms = self._time_grouped()
        except AccfftError:
            pass                        # a length without grouped kernels
        if grouped_ms is not None and grouped_ms < times[self.streams]:
            self.form = "grouped"
        else:
            self.form = "streams"
        if self.cache:
            json.dump(cached, open(self.cache, "w"), indent=1)
        return {"schedule": {"x".join(map(str, s)): v for s, v in self.schedule.items()},
                "streams": self.streams, "stream_ms": times, "grouped_ms": grouped_ms, "form": self.form}

    def report(self):
        rows = []
        for shape in sorted({i.shape for i in self.instances}):
            axes = {"x": radix_plan(shape[0], self.dtype), "y": radix_plan(shape[1], self.dtype),
                    "z_half": radix_plan(shape[2] // 2, self.dtype)}
            inst = next(i for i in self.instances if i.shape == shape)
            rows.append({"grid": list(shape), "schedule": self.schedule.get(shape, "split"), "radix": axes,
                         "tuned_passes": inst.plan.tuning() if inst.plan is not None else None})
        return rows

    # ------------------------------------------------------- grouped form
    def grouped(self):
        """The recorded, level-by-level form of the batch (built once)."""
        if self._batch is None:
            b = Batch()
            for inst in self.instances:
                if inst.plan is None or self.schedule.get(inst.shape, "split") != "split":
                    inst.make_plan("split")
                with b.recording(inst.plan):
                    inst.enqueue(torch.cuda.current_stream())
            b.finalize()
            self._batch = b
        return self._batch

    def _time_grouped(self, reps=3):
        b = self.grouped()
        main = torch.cuda.current_stream()
        b.run(main)
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(main)
        for _ in range(reps):
            b.run(main)
        e.record(main)
        torch.cuda.synchronize()
        return a.elapsed_time(e) / reps

    # ------------------------------------------------------------- capture
    def _enqueue_form(self, main):
        if self.form == "grouped":
            self.grouped().run(main)
        else:
            self._enqueue_all(main, self.streams)

    def capture(self):
        # every kernel and shared-memory attribute is set up by an eager run
        torch.cuda.synchronize()
        self._enqueue_form(torch.cuda.current_stream())
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        # relaxed: the plans query pointer attributes while enqueuing
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self._enqueue_form(torch.cuda.current_stream())
        torch.cuda.synchronize()

    def run(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
