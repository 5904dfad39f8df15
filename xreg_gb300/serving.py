"""Continuous-batching registration server.

Requests (a `Registration`: volume, cameras, fixed images per level, initial
pose, optimizer schedule) arrive at any time.  Each server step:

  1. admits queued jobs in arrival order while the summed device footprint of
     the active and starting jobs stays within the HBM budget (their volumes
     are uploaded once and stay resident, as do fixed-image gradients and
     optimizer state); a job starts (volume upload, first level set-up) on a
     worker thread while the active jobs keep stepping, and joins the steps
     once it has started;
  2. samples every active job's population (CMA-ES sample or trust-region ask;
     a CMA-ES state in device memory is sampled inside the geometry launch and
     updated by the grad-NCC launch), evaluates all populations with one DRR
     launch over every job's (tile, pose) work and one batched grad-NCC launch,
     and updates every
     optimizer: one xr_regi_jobset_step call (native_step; otherwise the same
     steps driven from Python around one job-set evaluation);
  3. ends levels whose optimizer stopped (level change or completion) and
     retires finished jobs, recording their latency from arrival.

Because each job's optimizer has its own random stream and the job-set values
equal the values each job gets alone, a job's result does not depend on which
other jobs share its steps.
"""
from __future__ import annotations

import collections
import concurrent.futures
import time
from dataclasses import dataclass, field

import numpy as np

from . import api
from .regi import Registration


@dataclass
class ServerStats:
    completed: int = 0
    latencies_s: list = field(default_factory=list)   # arrival to completion
    queue_waits_s: list = field(default_factory=list)  # arrival to start (admission)
    services_s: list = field(default_factory=list)     # start to completion
    steps: int = 0
    poses_evaluated: int = 0
    busy_s: float = 0.0
    admit_s: float = 0.0  # steps spent waiting for a job start (nothing else to step)
    max_active: int = 0
    max_footprint: int = 0

    def summary(self) -> dict:
        lat = np.array(self.latencies_s) if self.latencies_s else np.zeros(1)
        wait = np.array(self.queue_waits_s) if self.queue_waits_s else np.zeros(1)
        serv = np.array(self.services_s) if self.services_s else np.zeros(1)
        return {"completed": self.completed, "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
                "queue_wait_p50_s": float(np.percentile(wait, 50)), "queue_wait_p99_s": float(np.percentile(wait, 99)),
                "service_p50_s": float(np.percentile(serv, 50)), "service_p99_s": float(np.percentile(serv, 99)),
                "steps": self.steps,
                "poses_evaluated": self.poses_evaluated, "busy_s": self.busy_s, "admit_s": self.admit_s,
                "max_active": self.max_active,
                "max_footprint_gb": self.max_footprint / 1e9}


class RegistrationServer:
    def __init__(self, device: int = -1, hbm_budget_bytes: float = 180e9, max_active: int = 64,
                 native_step: bool = True, device_optimizer: bool = True):
        self.device = device
        # native_step: each generation of all active jobs (sample, evaluate,
        # update, stop test) in one library call; otherwise driven from Python
        self.native_step = bool(native_step)
        # device_optimizer (native steps only): CMA-ES levels keep their state in
        # device memory and are sampled and updated inside the step's launches
        self.device_optimizer = bool(device_optimizer) and self.native_step
        self.budget = float(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.queue: collections.deque = collections.deque()
        self.active: list = []
        self.finished: list = []
        self.jobset = api.JobSet(device)
        self.stats = ServerStats()
        self.starting: list = []  # (job, future) of jobs starting on the worker thread
        self._pool = concurrent.futures.ThreadPoolExecutor(max_workers=1)

    def close(self) -> None:
        """Waits for job starts in flight and ends the worker thread."""
        self._pool.shutdown(wait=True)

    def submit(self, job: Registration, t_arrival: float | None = None) -> None:
        job.t_submit = time.perf_counter() if t_arrival is None else t_arrival
        self.queue.append(job)

    def footprint(self) -> int:
        return sum(j.footprint_bytes() for j in self.active) + sum(j.footprint_bytes() for j, _ in self.starting)

    def _admit(self) -> None:
        used = self.footprint()
        while self.queue and len(self.active) + len(self.starting) < self.max_active:
            need = self.queue[0].footprint_bytes()
            if (self.active or self.starting) and used + need > self.budget:
                break
            job = self.queue.popleft()
            job.device_optimizer = self.device_optimizer
            self.starting.append((job, self._pool.submit(job.start)))
            used += need
        self.stats.max_footprint = max(self.stats.max_footprint, used)
        # started jobs join the steps; with nothing to step, wait for the first start
        if self.starting and not self.active:
            t0 = time.perf_counter()
            concurrent.futures.wait([self.starting[0][1]])
            self.stats.admit_s += time.perf_counter() - t0
        still = []
        for job, fut in self.starting:
            if fut.done():
                fut.result()  # a failed start raises here
                self.active.append(job)
            else:
                still.append((job, fut))
        self.starting = still
        self.stats.max_active = max(self.stats.max_active, len(self.active))

    def step(self) -> int:
        """One optimizer generation for every active job; returns the number of jobs stepped."""
        self._admit()
        if not self.active:
            return 0
        t0 = time.perf_counter()
        jobs = list(self.active)
        if self.native_step:
            stop, evaluated = self.jobset.regi_step([j.step_job() for j in jobs])
            for j, code in zip(jobs, stop):
                if code:
                    j.end_level(j.stop_reason(code))
            n_eval = sum(evaluated)
        else:
            poses = [j.propose() for j in jobs]
            values = self.jobset.eval([j.obj for j in jobs], poses)
            for j, v in zip(jobs, values):
                j.tell(v)
            n_eval = sum(len(p) for p in poses)
        now = time.perf_counter()
        self.stats.busy_s += now - t0
        self.stats.steps += 1
        self.stats.poses_evaluated += n_eval
        still = []
        for j in jobs:
            if j.done:
                self.finished.append(j)
                self.stats.completed += 1
                self.stats.latencies_s.append(j.t_done - j.t_submit)
                self.stats.queue_waits_s.append(j.t_start - j.t_submit)
                self.stats.services_s.append(j.t_done - j.t_start)
            else:
                still.append(j)
        self.active = still
        return len(jobs)

    def run(self, arrivals=None) -> ServerStats:
        """Runs until every submitted job is done.  arrivals: optional list of
        (offset_seconds, Registration) released when the wall clock passes them."""
        pending = sorted(arrivals or [], key=lambda a: a[0])
        t0 = time.perf_counter()
        i = 0
        while i < len(pending) or self.queue or self.active or self.starting:
            now = time.perf_counter() - t0
            while i < len(pending) and pending[i][0] <= now:
                self.submit(pending[i][1], t0 + pending[i][0])
                i += 1
            if not self.queue and not self.active and not self.starting:
                time.sleep(max(0.0, min(0.01, pending[i][0] - now)) if i < len(pending) else 0.0)
                continue
            self.step()
        return self.stats
