"""Request serving on one GPU: resident meshes, HBM-footprint admission,
continuous batching of independent solves.

A request is one 3D P3 SIP-DG Poisson solve: a mesh size (one of the
resident Kuhn-cube meshes), a per-element diffusivity kappa and a nodal
source f; the answer is the FP64 solution to ||b - A x|| <= rtol ||b||
(mixed-precision solve).  Per-request kappa changes the operator, so a
request rebuilds the operator blocks, the Galerkin P1CG operator, the SFC
level values and the mixed-precision copies in its slot before solving.

* Resident state: per mesh size the host mesh, its SFC ordering and a pool
  of slots; a slot is one library context (``DGSolver``) with every device
  buffer of a solve on that mesh, created once and reused.
* Admission by HBM footprint: the footprint of a mesh's slot is taken when
  its first slot is set up (the device bytes the library allocated for the
  context through set-up, build and one warm solve, plus the request's
  vectors and an allowance for streams and graphs); a new slot is created
  only while the sum of the slots' footprints stays within ``hbm_budget``; a
  request waits (FIFO) until a slot of its mesh is free or can be created.
* Continuous batching: requests that arrive while others run are admitted
  as soon as a slot frees up or fits; every admitted request runs on its own
  CUDA stream from its own host thread (the library releases the GIL inside
  its calls), so the solves of different requests overlap on the device.
* Each slot's computation depends only on its request (deterministic
  fixed-order reductions, no shared device state), so a result is the same
  alone and in the mix.

The reference has no serving layer; this module is the host side of the
batched/served form of the solve.
"""
from __future__ import annotations

import dataclasses
import threading
import time
from typing import Dict, List, Optional

import numpy as np

from . import element, mesh as mesh_mod, sfc
from .solver import DGSolver, SolverConfig


def _torch():
    import torch
    return torch


@dataclasses.dataclass
class Request:
    rid: int
    n: int                       # cells per cube side of the mesh
    kappa: np.ndarray            # (nele,) per-element diffusivity
    f: np.ndarray                # (nele * 20,) nodal source
    arrival: float = 0.0         # seconds after the start of the run


@dataclasses.dataclass
class Result:
    rid: int
    n: int
    x: np.ndarray                # FP64 solution, (nele * 20,)
    its: int                     # inner iterations
    residual: float              # final ||b - A x||
    tol: float
    arrival: float
    start: float                 # admission time
    end: float                   # completion time (solution on the host)
    build_s: float = 0.0         # operator rebuild for the request's kappa
    solve_s: float = 0.0         # mixed solve (incl. its reduced-precision copies and coarse inverse)

    @property
    def latency(self) -> float:
        return self.end - self.arrival


class _Slot:
    def __init__(self, solver: DGSolver):
        torch = _torch()
        self.solver = solver
        self.stream = torch.cuda.Stream(device=solver.cfg.device)
        self.busy = False


class SolveServer:
    """Continuous-batching server for SIP-DG solves on resident meshes."""

    def __init__(self, sizes, hbm_budget: float, rtol: float = 1e-10, face_kappa: str = "harmonic",
                 smooth: int = 2, device: int = 0, max_slots_per_size: int = 8, seed: int = 0,
                 dense_max: int = 1200):
        self.sizes = list(sizes)
        self.hbm_budget = float(hbm_budget)
        self.rtol = rtol
        self.face_kappa = face_kappa
        self.device = device
        self.max_slots = max_slots_per_size
        # exact coarse solve size of the mixed preconditioner: its inverse is
        # rebuilt per request (Gauss-Jordan, cost ~ rows^3), so a serving slot
        # keeps it smaller than the library default
        self.dense_max = dense_max
        self.cfg = SolverConfig(pre_smooth_its=smooth, post_smooth_its=smooth, device=device)
        self.meshes = {}
        self.orders = {}
        for n in self.sizes:
            m = mesh_mod.build_mesh("tet", n, seed=seed)
            self.meshes[n] = m
            self.orders[n] = sfc.hilbert_sfc_order(m.cg_coords)
        self.el = element.p3_element(3)
        self.slots: Dict[int, List[_Slot]] = {n: [] for n in self.sizes}
        self.footprint: Dict[int, float] = {}
        self.used = 0.0
        self._lock = threading.Condition()

    # -- slots ------------------------------------------------------------
    # device memory of a slot beyond what its library context allocates: the
    # context's streams and captured CUDA graphs
    GRAPH_ALLOWANCE = 64 << 20

    def _new_slot(self, n: int) -> _Slot:
        torch = _torch()
        s = DGSolver(self.meshes[n], self.orders[n], self.cfg, self.el)
        s.set_mixed_options(dense_max=self.dense_max)
        # every request rebuilds the operator: the affine block build (equal
        # to the quadrature build within 1e-13) keeps that rebuild short
        s.set_build_mode("affine")
        slot = _Slot(s)
        if n not in self.footprint:
            # warm set-up on a unit-kappa problem measures the slot's footprint
            with torch.cuda.stream(slot.stream):
                s.set_face_kappa(self.face_kappa)
                s.build_operator()
                b = s.rhs(torch.ones(s.nonods, dtype=torch.float64, device=s._dev()))
                x = torch.zeros_like(b)
                s.solve_mixed(x, b, 1e-6 * float(torch.linalg.norm(b)))
            slot.stream.synchronize()
            # the library reports its own allocations for the context, so
            # slots of other meshes allocating at the same time do not enter
            # the figure; add the request's vectors (f, b, x) and the graphs
            self.footprint[n] = float(s.info()["device_bytes"] + 3 * 8 * s.nonods + self.GRAPH_ALLOWANCE)
        self.used += self.footprint[n]
        self.slots[n].append(slot)
        return slot

    def _acquire(self, n: int) -> Optional[_Slot]:
        for slot in self.slots[n]:
            if not slot.busy:
                slot.busy = True
                return slot
        need = self.footprint.get(n)
        if len(self.slots[n]) < self.max_slots and (need is None or self.used + need <= self.hbm_budget
                                                     or not self.slots[n]):
            slot = self._new_slot(n)
            slot.busy = True
            return slot
        return None

    def prewarm(self, slots_per_size: Dict[int, int]):
        """Create slots ahead of traffic (as a deployment would), within the
        HBM budget: ``slots_per_size[n]`` slots for mesh size n."""
        for n, k in slots_per_size.items():
            while len(self.slots[n]) < min(k, self.max_slots):
                need = self.footprint.get(n)
                if need is not None and self.used + need > self.hbm_budget and self.slots[n]:
                    break
                self._new_slot(n)

    # -- one request ------------------------------------------------------
    def solve_one(self, slot: _Slot, req: Request):
        """Rebuild the slot's operator for the request's kappa and solve."""
        torch = _torch()
        s = slot.solver
        t0 = time.perf_counter()
        with torch.cuda.stream(slot.stream):
            s.set_kappa(req.kappa)
            s.set_face_kappa(self.face_kappa)
            s.build_operator()
            f = torch.tensor(req.f, dtype=torch.float64).pin_memory().to(s._dev(), non_blocking=True)
            b = s.rhs(f)
            x = torch.zeros_like(b)
            tol = self.rtol * float(torch.linalg.norm(b))
            t1 = time.perf_counter()
            its, res, _ = s.solve_mixed(x, b, tol)
            xh = x.cpu()
        slot.stream.synchronize()
        t2 = time.perf_counter()
        return xh.numpy(), its, res, tol, t1 - t0, t2 - t1

    # -- the serving loop ---------------------------------------------------
    def run(self, requests: List[Request]) -> List[Result]:
        """Serve the requests at their arrival times (seconds from now)."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        results: List[Result] = []
        pending: List[Request] = []
        threads = []
        errors = []
        t0 = time.perf_counter()
        i = 0

        def worker(slot: _Slot, req: Request, start: float):
            try:
                x, its, res, tol, tb, ts = self.solve_one(slot, req)
                end = time.perf_counter() - t0
                with self._lock:
                    results.append(Result(req.rid, req.n, x, its, res, tol, req.arrival, start, end, tb, ts))
            except Exception as exc:  # reported after the run
                with self._lock:
                    errors.append((req.rid, exc))
            finally:
                with self._lock:
                    slot.busy = False
                    self._lock.notify_all()

        with self._lock:
            while i < len(reqs) or pending or any(th.is_alive() for th in threads):
                now = time.perf_counter() - t0
                while i < len(reqs) and reqs[i].arrival <= now:
                    pending.append(reqs[i])
                    i += 1
                # admit in arrival order; a request whose mesh has no slot
                # available does not block requests for other meshes
                still = []
                for req in pending:
                    slot = self._acquire(req.n)
                    if slot is None:
                        still.append(req)
                        continue
                    th = threading.Thread(target=worker, args=(slot, req, time.perf_counter() - t0), daemon=True)
                    threads.append(th)
                    th.start()
                pending = still
                threads = [th for th in threads if th.is_alive()]
                wait = 0.05
                if i < len(reqs):
                    wait = max(0.0, min(wait, reqs[i].arrival - (time.perf_counter() - t0)))
                if pending or i < len(reqs) or threads:
                    self._lock.wait(timeout=wait if wait > 0 else 0.001)
        if errors:
            raise RuntimeError("request %d failed: %r" % errors[0])
        return sorted(results, key=lambda r: r.rid)

    def close(self):
        for n in self.slots:
            for slot in self.slots[n]:
                slot.solver.close()
            self.slots[n] = []
        self.used = 0.0


def make_requests(sizes, count: int, rate: float, sigma: float = 0.5, seed: int = 0,
                  meshes: Optional[dict] = None) -> List[Request]:
    """Seeded request stream: mesh size drawn uniformly from ``sizes``,
    per-element log-normal kappa exp(sigma N(0,1)), an 8-mode Fourier source
    (integer wavenumbers 1..4, N(0,1) amplitudes), Poisson arrivals at
    ``rate`` per second (exponential gaps)."""
    rng = np.random.default_rng(seed)
    meshes = meshes or {n: mesh_mod.build_mesh("tet", n, seed=0) for n in sorted(set(sizes))}
    reqs = []
    t = 0.0
    for rid in range(count):
        n = int(rng.choice(sizes))
        m = meshes[n]
        kappa = np.exp(sigma * rng.standard_normal(m.nele))
        X = m.x_ref_in
        f = np.zeros((m.nele, m.nloc))
        for _ in range(8):
            k = rng.integers(1, 5, size=3)
            a = rng.standard_normal()
            f += a * np.pi ** 2 * float((k ** 2).sum()) * np.prod([np.sin(k[d] * np.pi * X[:, d]) for d in range(3)],
                                                                axis=0)
        f *= kappa[:, None]
        reqs.append(Request(rid, n, kappa, f.reshape(-1), arrival=t))
        t += rng.exponential(1.0 / rate)
    return reqs


def latency_stats(results: List[Result]) -> dict:
    lat = np.array([r.latency for r in results])
    span = max(r.end for r in results) - min(r.arrival for r in results)
    dofs = sum(r.x.size for r in results)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "requests": len(results), "span_s": float(span),
            "dofs_per_s": float(dofs / span),
            "mean_build_s": float(np.mean([r.build_s for r in results])),
            "mean_solve_s": float(np.mean([r.solve_s for r in results])),
            "mean_wait_s": float(np.mean([r.start - r.arrival for r in results]))}


class NativeQueue:
    """The library's own request queue (dg_server_create / dg_enqueue /
    dg_poll / dg_wait in include/dgsip.h): ``nworkers`` native threads with
    one CUDA stream each run queued solves on ``DGSolver`` contexts, one
    request per context at a time, in arrival order per context.  A request
    may carry a new per-element kappa: the worker rebuilds the context's
    operator with it before solving.  x and b (FP64 CUDA tensors) are kept
    referenced here until the request is reported done; the caller must not
    use the solver in the meantime, and must have finished writing x and b
    (e.g. torch.cuda.synchronize()) before enqueueing: the workers' streams
    do not wait for the caller's."""

    def __init__(self, nworkers: int = 2, device: int = 0):
        import ctypes as C
        from . import _capi
        self._C = C
        self._capi = _capi
        self._lib = _capi.lib()
        h = C.c_void_p()
        _capi.check(self._lib.dg_server_create(int(device), int(nworkers), C.byref(h)))
        self._h = h
        self._keep: Dict[int, tuple] = {}

    def enqueue(self, solver: DGSolver, x, b, tol: float, mode: str = "mixed", m: Optional[int] = None,
                max_its: Optional[int] = None, inner_rtol: float = 1e-3, kappa: Optional[np.ndarray] = None) -> int:
        C = self._C
        if mode not in ("mixed", "fp64"):
            raise ValueError("mode must be 'mixed' or 'fp64'")
        k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        if k is not None and k.size != solver.mesh.nele:
            raise ValueError("kappa needs one value per element")
        rid = C.c_int64(0)
        self._capi.check(self._lib.dg_enqueue(
            self._h, solver._ctx, solver._check_t(x, solver.nonods), solver._check_t(b, solver.nonods), float(tol),
            0 if mode == "mixed" else 1, int(m if m is not None else solver.cfg.gmres_m),
            int(max_its if max_its is not None else solver.cfg.gmres_its), float(inner_rtol),
            None if k is None else k.ctypes.data, C.byref(rid)))
        self._keep[rid.value] = (x, b, k, solver)
        return rid.value

    def _report(self, fn, rid, *args):
        C = self._C
        st, status, its = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        res = C.c_double(0.0)
        secs = (C.c_double * 2)()
        self._capi.check(fn(self._h, C.c_int64(rid), *args, C.byref(st), C.byref(status), C.byref(its),
                            C.byref(res), C.cast(secs, C.c_void_p)))
        if st.value != self._capi.DG_REQ_DONE:
            return None
        self._keep.pop(rid, None)
        return {"status": status.value, "its": its.value, "res": res.value, "wait_s": secs[0], "run_s": secs[1]}

    def poll(self, rid: int):
        """None while queued or running; once done, a dict with the solve's
        return code ("status"), its, res, wait_s and run_s (reported once)."""
        return self._report(self._lib.dg_poll, rid)

    def wait(self, rid: int, timeout: float = -1.0):
        """poll() after waiting up to ``timeout`` seconds (< 0: no limit)."""
        return self._report(self._lib.dg_wait, rid, self._C.c_double(float(timeout)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.dg_server_destroy(self._h)
            self._h = self._C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
