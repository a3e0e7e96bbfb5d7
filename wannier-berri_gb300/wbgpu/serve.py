"""Continuous-batching integration server: resident systems, concurrent requests.

The reference integrates one system per ``run()`` call (run_grid.py:118-403) and leaves
concurrency to Ray processes (run_grid.py:79-109).  This module keeps many systems resident on
one GPU and runs many integration requests at once:

* ``Server.add_system`` uploads a system's R-space matrices once (engine.DeviceSystem); the
  k-independent R-space fields and grid phase tables are built on first use and cached.
* ``Server.submit`` queues a request (system, grid, calculators[, blocks]) and returns a
  ``Ticket``.  Requests are admitted in arrival order while an active slot is free and the
  request's estimated device memory fits in the HBM budget; nothing overtakes the queue head.
* Every admitted request gets its own CUDA stream and buffer workspace, and its Fermi-level
  histograms stay on the device.  The scheduler issues one block batch per active request per
  round, so kernels of different requests overlap on the GPU; a request's completion is seen
  through an event on its stream (no device-wide synchronisation).
* Results are the same ``ResultDict`` as ``run()`` with the same block weighting; ``stats()``
  reports p50 / p99 latency (submit to result) and k-points per second.
* A request with ``adpt_num_iter`` > 0 runs in rounds of adaptive refinement (run.Refinement,
  the reference's policy): each round's blocks get per-block results; when the round's event
  fires, the host selects and divides K-points and queues the next round on the same stream.
* A request with ``refine_omega`` > 0 runs in rounds of refinement around the largest Berry
  curvatures (run.OmegaRefinement): every batch also writes its k-points' max_n |Omega_n(k)|;
  when a round's event fires, the host takes the top fraction and queues their sub-grids.

No counterpart in the reference; the numerical path is exactly ``run()``'s.
"""
import copy
import threading
import time
from collections import deque

import numpy as np
import torch

from . import engine
from .result import ResultDict
from .run import OmegaRefinement, Refinement, _omega_scores, choose_batch


def admit(pending_bytes, used_bytes, budget_bytes, free_slots):
    """Admission rule: the longest prefix of the FIFO queue (sizes `pending_bytes`) that fits
    in the free slots and the remaining memory budget.  Returns the number admitted.  A request
    larger than the whole budget is admitted alone when nothing else is active (it could never
    run otherwise)."""
    n = 0
    for size in pending_bytes:
        if n >= free_slots:
            break
        if used_bytes + size > budget_bytes and not (used_bytes == 0 and n == 0):
            break
        used_bytes += size
        n += 1
    return n


def later_batch_of_size(batches, start, size):
    """Whether a batch of `size` blocks is among batches[start:] (block-index arrays)."""
    return any(len(b) == size for b in batches[start:])


def request_bytes(nw, nk, nblocks_batch, quantities, precision):
    """Device memory of one request's batch buffers (fields, H, U, Xbar, workspaces)."""
    cs = 16 if precision == 'fp64' else 8
    nf = 1 + sum(engine.QUANTITIES[q]['ncomp'] for q in quantities)
    per_k = nw * nw * (2 * nf * cs + 16 * 3) + 64 * nw
    return int(per_k * nk * nblocks_batch * 2)


class Ticket:
    """Handle of a submitted request: ``wait()`` returns its ResultDict (or raises its error)."""

    def __init__(self, rid, key):
        self.rid, self.key = rid, key
        self.t_submit = time.perf_counter()
        self.t_admit = None
        self.t_done = None
        self.nkpoints = 0
        self._event = threading.Event()
        self._result = None
        self._error = None

    def done(self):
        return self._event.is_set()

    def wait(self, timeout=None):
        if not self._event.wait(timeout):
            raise TimeoutError(f"request {self.rid} not finished after {timeout} s")
        if self._error is not None:
            raise self._error
        return self._result

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    def _finish(self, result=None, error=None):
        self.t_done = time.perf_counter()
        self._result, self._error = result, error
        self._event.set()


class _Request:
    def __init__(self, ticket, key, grid, calculators, blocks, adapt=None, omega=None):
        self.ticket, self.key, self.grid, self.calculators = ticket, key, grid, calculators
        self.blocks = blocks
        self.adapt = adapt  # (adpt_num_iter, adpt_mesh, adpt_fac) or None
        self.refine = None  # run.Refinement of an adaptive request
        self.omega = omega  # (rounds, top, mesh) of a refinement around the largest |Omega|, or None
        self.oref = None  # its run.OmegaRefinement
        self.ophases = None  # phase tables of the round's jobs (and their staging buffers)
        self.score_parts = []
        self.shifts = None  # block shifts of the current round (adaptive requests)
        self.cells = None  # and their dense-grid cells
        self.round_calcs = []
        self.stream = None
        self.ws = None
        self.batches = None
        self.next_batch = 0
        self.done_event = None
        self.nbytes = 0
        self.flags = []


class Server:
    """Continuous-batching server on one device.

    precision: 'mixed' or 'fp64' (as run()); hbm_budget: bytes of per-request buffers allowed
    at once; max_active: requests in flight (one CUDA stream each); max_kpoints: k-points per
    block batch; cuda_graph: replay stages 1-3 of a request's batches from CUDA graphs
    (engine.band_data_graphed, one set per request workspace); autotune: launch shapes of each
    resident system's num_wann from the autotuner (wbgpu.autotune.ensure, at add_system)."""

    def __init__(self, device='cuda', precision='mixed', hbm_budget=150 << 30, max_active=4, max_kpoints=1 << 17,
                 cuda_graph=False, autotune=False):
        engine.require_cuda()
        self.device = torch.device(device)
        self.precision = precision
        self.cuda_graph = bool(cuda_graph)
        self.autotune = bool(autotune)
        self._tuned = set()
        self.hbm_budget = int(hbm_budget)
        self.max_active = int(max_active)
        self.max_kpoints = int(max_kpoints)
        self._systems = {}
        self._pending = deque()
        self._active = []
        self._finished = []
        self._lock = threading.Lock()
        self._wake = threading.Event()
        self._stop = False
        self._thread = None
        self._rid = 0
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.max_active)]
        self._free_streams = list(self._streams)
        self._prep_stream = torch.cuda.Stream(device=self.device)
        self._used = 0
        self._error = None

    # ---------------------------------------------------------------- systems and requests
    def add_system(self, key, system):
        """Make `system` resident under `key` (R-space matrices uploaded now)."""
        with torch.cuda.stream(self._prep_stream):
            dev = engine.DeviceSystem(system, self.device)
            for name in ['Ham'] + [k for k in ('AA', 'BB', 'CC') if system.has_R_mat(k)]:
                dev._key_fp64(name)  # upload now: requests find the matrices resident
        self._prep_stream.synchronize()
        if self.autotune and dev.nw not in self._tuned:
            from . import autotune as _tune
            _tune.ensure(dev.nw, self.precision, device=self.device)
            self._tuned.add(dev.nw)
        self._systems[key] = (system, dev)
        return dev

    def submit(self, key, grid, calculators, blocks=None, adpt_num_iter=0, adpt_mesh=2, adpt_fac=1, refine_omega=0,
               refine_top=0.01, refine_mesh=8):
        """Queue an integration of `calculators` over `grid` (optionally a subset `blocks` of its
        division-grid K-points, with `adpt_num_iter` rounds of adaptive refinement, or with
        `refine_omega` rounds of refinement around the largest Berry curvatures: the `refine_top`
        fraction of the k-points by |Omega| refined by refine_mesh^3 sub-grids) for the system
        registered as `key`; returns a Ticket."""
        if key not in self._systems:
            raise ValueError(f"unknown system {key!r}: add_system() first")
        adapt = omega = None
        if adpt_num_iter:
            if blocks is not None:
                raise ValueError("adaptive refinement runs over the whole grid (blocks must be None)")
            adapt = (adpt_num_iter, adpt_mesh, adpt_fac)
        if refine_omega:
            if blocks is not None or adapt is not None:
                raise ValueError("refinement around |Omega| runs over the whole grid, without adpt_num_iter")
            omega = (int(refine_omega), float(refine_top), int(refine_mesh))
        with self._lock:
            self._rid += 1
            t = Ticket(self._rid, key)
            self._pending.append(_Request(t, key, grid, dict(calculators), blocks, adapt, omega))
        self._wake.set()
        return t

    # ---------------------------------------------------------------- scheduling
    def _estimate(self, req):
        system, dev = self._systems[req.key]
        q = set()
        for c in req.calculators.values():
            q |= c.quantities(system)
        nblk = len(self._blocks_of(req))
        nb = choose_batch(dev.nw, req.grid.nk_per_block, nblk, q, self.precision, max_kpoints=self.max_kpoints)
        nbytes = request_bytes(dev.nw, req.grid.nk_per_block, nb, q, self.precision)
        if self._tetra(req):  # resident corner energies of the tetrahedron method
            nbytes += engine.TetraCorners.nbytes(req.grid, nblk, dev.nw)
        return q, nb, nbytes

    @staticmethod
    def _tetra(req):
        return any(getattr(c, 'tetra', False) for c in req.calculators.values())

    @staticmethod
    def _blocks_of(req):
        shifts = req.grid.block_shifts()
        return np.arange(len(shifts)) if req.blocks is None else np.asarray(req.blocks)

    def _admit(self):
        with self._lock:
            sizes, plans = [], []
            for req in self._pending:
                if len(plans) >= len(self._free_streams):
                    break
                plan = self._estimate(req)
                plans.append(plan)
                sizes.append(plan[2])
            n = admit(sizes, self._used, self.hbm_budget, len(self._free_streams))
            taken = [self._pending.popleft() for _ in range(n)]
        for req, (q, nb, nbytes) in zip(taken, plans):
            self._start(req, q, nb, nbytes)

    def _start(self, req, quantities, nb, nbytes):
        system, dev = self._systems[req.key]
        req.ticket.t_admit = time.perf_counter()
        req.stream = self._free_streams.pop()
        req.nbytes = nbytes
        self._used += nbytes
        req.ws = engine.Workspace(self.device)
        blocks = self._blocks_of(req)
        shifts = req.grid.block_shifts()
        precs = engine.phase_precs(self.precision)
        # cached, k-independent data (R-space fields, phase tables) are built on the preparation
        # stream; the request's stream waits for them once
        with torch.cuda.stream(self._prep_stream):
            req.phases = {p: dev.grid_phases(shifts, req.grid.FFT, p) for p in precs}
            if self.precision == 'fp64':
                engine.field_arrays(dev, quantities, True, engine.PREC_FP64)
            else:
                engine.field_arrays(dev, set(), True, engine.PREC_DF64)
                if quantities:  # energies-only requests (DOS-type) need no band-basis fields
                    engine.field_arrays(dev, quantities, False, engine.MIXED_FIELDS_PREC)
            ready = torch.cuda.Event()
            ready.record(self._prep_stream)
        req.stream.wait_event(ready)
        req.quantities = quantities
        req.nb = nb
        if req.adapt is not None:
            req.refine = Refinement(system, req.grid, req.calculators, *req.adapt)
            self._plan_round(req)
        elif req.omega is not None:
            with torch.cuda.stream(req.stream):  # its calculators' buffers belong to the request's stream
                req.oref = OmegaRefinement(system, req.grid, req.calculators, self.device, *req.omega)
            req.quantities = req.oref.quantities
            req.ticket.nkpoints = 0
            self._plan_oround(req)
        else:
            req.batches = [blocks[i:i + nb] for i in range(0, len(blocks), nb)]
            req.ticket.nkpoints = len(blocks) * req.grid.nk_per_block
        with torch.cuda.stream(req.stream):
            for c in req.calculators.values():
                c.reset(self.device)
            req.tetra = None
            if self._tetra(req):
                req.tetra = engine.TetraCorners(dev, req.grid, blocks, self.precision, ws=req.ws)
                req.flags.extend(req.tetra.flags)
            if not req.batches:
                req.done_event = torch.cuda.Event()
                req.done_event.record(req.stream)
        self._active.append(req)

    def _plan_round(self, req):
        """Batches of the adaptive request's next round (the K-points not evaluated yet)."""
        req.shifts = req.refine.new_shifts()
        req.cells = req.refine.new_cells()
        n = len(req.shifts)
        req.batches = [np.arange(i, min(i + req.nb, n)) for i in range(0, n, req.nb)]
        req.next_batch = 0
        req.done_event = None
        req.ticket.nkpoints += n * req.grid.nk_per_block

    def _plan_oround(self, req):
        """Batches of the current round's jobs of a refinement around |Omega|: (job, blocks)."""
        system, dev = self._systems[req.key]
        req.batches, req.ophases = [], []
        for j, job in enumerate(req.oref.jobs()):
            n = len(job.shifts)
            nb = choose_batch(dev.nw, job.nk, n, req.quantities, self.precision, max_kpoints=self.max_kpoints)
            req.batches += [(j, np.arange(i, min(i + nb, n))) for i in range(0, n, nb)]
            with torch.cuda.stream(req.stream):
                if req.oref.round == 0:  # the grid itself: the system's cached tables
                    req.ophases.append(req.phases)
                else:
                    tabs = {}
                    for p in engine.phase_precs(self.precision):
                        tabs[p], host = dev.grid_phases(job.shifts, job.fft, p, step=job.step, cache=False)
                        tabs[(p, 'staging')] = host
                    req.ophases.append(tabs)
        req.ticket.nkpoints = req.oref.kpoints
        req.next_batch = 0
        req.done_event = None
        req.score_parts = []

    def _issue_omega(self, req, system, dev):
        j, idx = req.batches[req.next_batch - 1]
        job = req.oref.jobs()[j]
        ph = {p: t for p, t in req.ophases[j].items() if not isinstance(p, tuple)}
        bd = engine.band_data(dev, job.shifts[idx], job.fft, req.quantities, self.precision, phases=ph,
                              block_start=int(idx[0]), ws=req.ws)
        for c in job.calcs.values():
            c.accumulate(bd, system)
        if job.scores:
            req.score_parts.append(_omega_scores(bd, 1e-4).clone())
        return bd

    def _issue_adaptive(self, req, idx, system, dev):
        corners = None
        if any(getattr(c, 'tetra', False) for c in req.refine.templates.values()):
            corners = engine.BlockCorners(dev, req.shifts[idx], req.cells[idx], req.grid.FFT, self.precision,
                                          ws=req.ws)
            req.flags.extend(corners.flags)
        bd = engine.band_data(dev, req.shifts[idx], req.grid.FFT, req.quantities, self.precision, ws=req.ws)
        if corners is not None:
            corners.attach(bd, np.arange(bd.nblocks))
        for b in range(bd.nblocks):  # per-block results: fresh calculators for every block
            sub = bd.block(b)
            cs = {k: copy.deepcopy(c) for k, c in req.refine.templates.items()}
            for c in cs.values():
                c.reset(self.device)
                c.accumulate(sub, system)
            req.round_calcs.append(cs)
        return bd

    def _end_round(self, req):
        """The round's kernels are done: per-block results, then the next round or the end."""
        system, dev = self._systems[req.key]
        with torch.cuda.stream(req.stream):
            nk = req.grid.nk_per_block
            req.refine.add([{k: c.result(system.cell_volume, nk, 1.0) for k, c in cs.items()}
                            for cs in req.round_calcs])
        req.round_calcs = []
        if req.refine.refine():
            self._plan_round(req)
            return False
        return True

    def _end_oround(self, req):
        """A round of a refinement around |Omega| is done: add its results, plan the next."""
        with torch.cuda.stream(req.stream):
            scores = torch.cat(req.score_parts) if req.score_parts else None
            more = req.oref.end_round(scores)
        if more:
            self._plan_oround(req)
            return False
        return True

    def _issue(self, req):
        system, dev = self._systems[req.key]
        idx = req.batches[req.next_batch]
        req.next_batch += 1
        shifts = req.grid.block_shifts()
        if req.oref is not None:
            with torch.cuda.stream(req.stream):
                bd = self._issue_omega(req, system, dev)
                req.flags.append(bd._flag.clone())
                if req.next_batch == len(req.batches):
                    req.done_event = torch.cuda.Event()
                    req.done_event.record(req.stream)
            return
        with torch.cuda.stream(req.stream):
            contiguous = np.all(np.diff(idx) == 1)
            stages = engine.band_data
            if self.cuda_graph:  # capture only when a later batch of this request has the same size
                more = later_batch_of_size(req.batches, req.next_batch, len(idx))
                stages = lambda *a, **k: engine.band_data_graphed(*a, more=more, **k)
            if req.refine is not None:
                bd = self._issue_adaptive(req, idx, system, dev)
            elif contiguous:
                bd = stages(dev, shifts[idx], req.grid.FFT, req.quantities, self.precision,
                            phases=req.phases, block_start=int(idx[0]), ws=req.ws)
            else:
                bd = stages(dev, shifts[idx], req.grid.FFT, req.quantities, self.precision, ws=req.ws)
            if req.tetra is not None:
                req.tetra.attach(bd, idx)
            for c in req.calculators.values():
                c.accumulate(bd, system)
            # the QL convergence flag is read once the request has finished
            req.flags.append(bd._flag.clone())
            if req.next_batch == len(req.batches):
                req.done_event = torch.cuda.Event()
                req.done_event.record(req.stream)

    def _finish(self, req):
        system, dev = self._systems[req.key]
        try:
            with torch.cuda.stream(req.stream):
                if any(int(f.item()) != 0 for f in req.flags):
                    raise RuntimeError("wbg_eigh_batched: QL iteration did not converge for some k-point")
                nk = req.grid.nk_per_block
                factor = 1.0 / req.grid.nblocks
                if req.refine is not None:
                    res = req.refine.total()
                elif req.oref is not None:
                    res = req.oref.result()
                else:
                    res = ResultDict({k: c.result(system.cell_volume, nk, factor)
                                      for k, c in req.calculators.items()})
            req.ticket._finish(result=res)
        except Exception as e:  # the request fails, the server keeps going
            req.ticket._finish(error=e)
        req.ws.release()
        self._used -= req.nbytes
        self._free_streams.append(req.stream)
        self._finished.append(req.ticket)

    def _fail(self, req, error):
        """Retire a request whose issue or round end raised: its ticket gets the error, its work
        already queued on its stream is waited for before its buffers and stream are reused, and
        the other requests go on."""
        if req in self._active:
            self._active.remove(req)
        try:
            req.stream.synchronize()
        finally:
            req.ticket._finish(error=error)
            req.ws.release()
            self._used -= req.nbytes
            self._free_streams.append(req.stream)
            self._finished.append(req.ticket)

    def step(self):
        """One scheduler round: admit, issue one batch per active request, retire finished
        requests.  A request whose work raises on the host (a calculator, a refinement round)
        fails alone.  Returns True while there is work left."""
        self._admit()
        for req in list(self._active):
            if req.next_batch < len(req.batches):
                try:
                    self._issue(req)
                except Exception as e:
                    self._fail(req, e)
        for req in list(self._active):
            if req.next_batch == len(req.batches) and req.done_event.query():
                if req.refine is not None or req.oref is not None:
                    try:
                        if not (self._end_round(req) if req.refine is not None else self._end_oround(req)):
                            continue  # next refinement round queued on the same stream
                    except Exception as e:
                        self._fail(req, e)
                        continue
                self._active.remove(req)
                self._finish(req)
        with self._lock:
            return bool(self._pending or self._active)

    def run_until_idle(self, poll=0.0002):
        """Drive the scheduler in the calling thread until every submitted request is done."""
        while self.step():
            if all(r.next_batch == len(r.batches) for r in self._active):
                time.sleep(poll)

    # ---------------------------------------------------------------- background thread
    def _loop(self):
        try:
            while not self._stop:
                if not self.step():
                    self._wake.wait(0.01)
                    self._wake.clear()
                elif all(r.next_batch == len(r.batches) for r in self._active):
                    time.sleep(0.0002)
        except Exception as e:  # surface scheduler failures to every waiting ticket
            self._error = e
            with self._lock:
                reqs = list(self._pending) + list(self._active)
                self._pending.clear()
            for r in reqs:
                r.ticket._finish(error=e)

    def start(self):
        if self._thread is None:
            self._stop = False
            self._thread = threading.Thread(target=self._loop, name="wbgpu-server", daemon=True)
            self._thread.start()
        return self

    def stop(self):
        self._stop = True
        self._wake.set()
        if self._thread is not None:
            self._thread.join()
            self._thread = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # ---------------------------------------------------------------- statistics
    def stats(self, tickets=None):
        """Latency percentiles (ms) and throughput over finished tickets."""
        ts = [t for t in (tickets if tickets is not None else self._finished) if t.t_done is not None]
        if not ts:
            return {"requests": 0}
        lat = np.array([t.latency for t in ts]) * 1e3
        t0 = min(t.t_submit for t in ts)
        t1 = max(t.t_done for t in ts)
        nk = sum(t.nkpoints for t in ts)
        return {"requests": len(ts), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max()), "kpoints": int(nk), "kpoints_per_s": nk / max(t1 - t0, 1e-9)}


def run_many(jobs, precision='mixed', max_active=4, device='cuda', cuda_graph=False, autotune=False):
    """Integrate a list of (system, grid, calculators) jobs concurrently through one Server
    (systems made resident once); returns the list of ResultDicts in job order."""
    srv = Server(device=device, precision=precision, max_active=max_active, cuda_graph=cuda_graph,
                 autotune=autotune)
    keys = {}
    tickets = []
    for system, grid, calcs in jobs:
        if id(system) not in keys:
            keys[id(system)] = len(keys)
            srv.add_system(keys[id(system)], system)
        tickets.append(srv.submit(keys[id(system)], grid, calcs))
    srv.run_until_idle()
    return [t.wait() for t in tickets]
