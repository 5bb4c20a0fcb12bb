"""Many independent interface problems of uneven size trained together.

Each instance has its own level set, residual records, network parameters, Adam state and step
workspace (the reference trains one problem per ``Trainer``; examples/benchmark_LPBE runs its
molecules one by one).  ``InstanceBatch`` trains them together and captures the batched step in
one CUDA graph, so that a batched step is one graph launch.

For the tile-engine shapes (3x32, 2x16) the step is ``dips_train_step_instances``: one launch
per phase for all instances over a device table of the instances (batch ids, expansion, general
forward, general residual, training launch, gradient tail), the two tile-engine launches
persistent over every instance's tiles.  Other shapes run one ``dips_train_step`` per instance,
dealt largest first over several capture streams, which the GPU runs side by side.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, levelset, mesh, nn, ops
from .records import FVLevel

F32 = np.float32


class Instance:
    """One problem: its grid, level set, records at h = dx, parameters and optimizer."""

    def __init__(self, side: int, problem: dict, arch: nn.Arch, batch: int, lr: float, seed: int, device="cuda"):
        self.side = side
        self.grid = mesh.uniform_grid(side)
        g = self.grid
        self.ls = levelset.LevelSetGrid.from_callable(g, lambda r: levelset.perturb(problem["phi"](r)), device)
        pts = torch.as_tensor(g.R, device=device)
        self.level = FVLevel(self.ls, problem, pts, np.array([g.dx, g.dy, g.dz], F32))
        self.batch = min(int(batch), self.level.n)
        self.n_batches = self.level.n // self.batch
        self.params = torch.as_tensor(nn.init_params(arch, seed), device=device)
        self.opt = ops.AdamState(nn.n_params(arch), lr=lr, decay_rate=0.9, device=device)
        self.ws = ops.StepWorkspace(arch, self.batch, self.level.max_jobs(self.batch), device)
        self.ids = torch.empty(self.batch, dtype=torch.int32, device=device)
        self.loss = torch.zeros((), dtype=torch.float64, device=device)
        self.seed = seed


class InstanceBatch:
    """Train ``len(instances)`` problems with one graph launch per batched step.

    instances: list of (grid side, problem dict).  batch: points per instance and step (clamped
    to the instance's size); minibatches are uniform permutations per epoch of each instance.
    """

    def __init__(self, instances, arch: nn.Arch, batch: int = 1 << 15, lr: float = 1e-3, seed: int = 0,
                 device="cuda", streams: int = 8, persistent=None, autotune: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("dips_gb300 runs on a CUDA GPU; none is available")
        lib = _lib.load()
        if not lib.dips_arch_supported(arch.ctype()):
            raise NotImplementedError(lib.dips_last_error().decode())
        self.arch = arch
        self.device = device
        self.items = [Instance(side, prob, arch, batch, lr, seed + i, device) for i, (side, prob) in enumerate(instances)]
        self.order = sorted(range(len(self.items)), key=lambda i: -self.items[i].level.n)
        self.losses = torch.zeros(len(self.items), dtype=torch.float64, device=device)
        self.streams = [torch.cuda.Stream(device=device) for _ in range(max(1, int(streams)))]
        self.graph = None
        tile = (arch.m_layers, arch.m_width) == (arch.p_layers, arch.p_width) and \
            (arch.m_layers, arch.m_width) in ((2, 16), (3, 32)) and arch.pre_layers == 0
        self.persistent = tile if persistent is None else bool(persistent)
        if self.persistent and not tile:
            raise NotImplementedError("the persistent multi-instance step needs a 3x32 or 2x16 shape")
        self.max_batch = max(it.batch for it in self.items)
        self._tables = {}
        self.cta_warps = 0
        if tile and autotune:
            # the tile engine's CTA width, timed on the largest instance (process-wide per device)
            big = self.items[self.order[0]]
            ids = ops.batch_ids(big.level.n, big.batch, epoch=0, batch_index=0, seed=big.seed, device=device)
            self.cta_warps = ops.autotune(arch, big.params, big.level, ids, big.ws)
        if self.persistent:
            self._table(ids_mode=1)

    def _table(self, ids_mode: int):
        """The device table of the instances (batch ids drawn on the device, ids_mode 1, or
        given by the caller, -1), prepared once."""
        if ids_mode in self._tables:
            return self._tables[ids_mode]
        lib = _lib.load()
        n = len(self.items)
        arr = (_lib.InstanceT * n)()
        for i, it in enumerate(self.items):
            arr[i] = _lib.InstanceT(
                ctypes.addressof(it.level.desc), _lib.ptr(it.ids), it.batch, it.n_batches, it.seed, ids_mode,
                _lib.ptr(it.params), _lib.ptr(it.opt.mu), _lib.ptr(it.opt.nu), _lib.ptr(it.opt.count),
                _lib.ptr(it.ws.buf), it.ws.nbytes, _lib.ptr(self.losses[i:i + 1]), None)
        nbytes = int(lib.dips_instances_table_bytes(n))
        table = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        _lib.check(lib.dips_instances_prepare(self.arch.ctype(), arr, n, _lib.ptr(table), nbytes,
                                              _lib.stream_handle()), "dips_instances_prepare")
        self._tables[ids_mode] = table
        return table

    def _step_persistent(self, ids_mode: int = 1):
        lib = _lib.load()
        _lib.check(lib.dips_train_step_instances(self.arch.ctype(), self.items[0].opt.hp,
                                                 _lib.ptr(self._table(ids_mode)), len(self.items), self.max_batch,
                                                 _lib.stream_handle()), "dips_train_step_instances")

    def step_with_ids(self):
        """One step of every instance on the batch ids already in each instance's ``ids`` (e.g.
        copied from the host), without a graph."""
        if self.persistent:
            self._step_persistent(ids_mode=-1)
            return self.losses
        for i in self.order:
            it = self.items[i]
            ops.train_step(self.arch, it.params, it.opt, it.level, it.ids, it.ws, it.loss)
            self.losses[i : i + 1].copy_(it.loss.reshape(1))
        return self.losses

    def _step_one(self, i):
        lib = _lib.load()
        it = self.items[i]
        _lib.check(lib.dips_batch_ids_device(it.level.n, it.batch, it.n_batches, it.seed, 1, _lib.ptr(it.opt.count),
                                             _lib.ptr(it.ids), _lib.stream_handle()), "dips_batch_ids_device")
        ops.train_step(self.arch, it.params, it.opt, it.level, it.ids, it.ws, it.loss)
        self.losses[i : i + 1].copy_(it.loss.reshape(1))

    def _step_all(self):
        """Every instance's step: the persistent multi-instance step, or one step per instance
        dealt over the side streams (fork from and join to the current stream, so that the whole
        batched step is ordered like one launch)."""
        if self.persistent:
            self._step_persistent()
            return
        main = torch.cuda.current_stream()
        for s in self.streams:
            s.wait_stream(main)
        for k, i in enumerate(self.order):
            with torch.cuda.stream(self.streams[k % len(self.streams)]):
                self._step_one(i)
        for s in self.streams:
            main.wait_stream(s)

    def capture(self):
        """Warm up once (restoring the state), then capture every instance's step in one graph."""
        saved = [(it.params.clone(), it.opt.mu.clone(), it.opt.nu.clone(), it.opt.count.clone()) for it in self.items]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._step_all()
        torch.cuda.current_stream().wait_stream(s)
        for it, (p, m, v, c) in zip(self.items, saved):
            it.params.copy_(p)
            it.opt.mu.copy_(m)
            it.opt.nu.copy_(v)
            it.opt.count.copy_(c)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._step_all()
        return self

    def step(self):
        """One training step of every instance (one graph launch once captured)."""
        if self.graph is None:
            self._step_all()
        else:
            self.graph.replay()
        return self.losses

    @property
    def points_per_step(self) -> int:
        return sum(it.batch for it in self.items)

    @property
    def kernels_per_step(self) -> int:
        """This library's kernel launches per batched step: per instance the batch ids, the
        expansion (3), the general forward, the general residual, the bulk training launch and
        the gradient tail (reduction, loss, Adam); shapes off the tile engine launch the forward,
        the bulk kernel and the adjoint once per network.  (A loss copy per instance is torch's.)"""
        if self.persistent:  # one launch per phase for all instances
            return 8
        a = self.arch
        tile = (a.m_layers, a.m_width) == (a.p_layers, a.p_width) and (a.m_layers, a.m_width) in ((2, 16), (3, 32))
        return (8 if tile else 12) * len(self.items)
