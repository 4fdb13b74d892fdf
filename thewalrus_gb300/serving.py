"""Continuous-batching server for Gaussian-state Fock probabilities on the GPU sieve.

A request is (state, photon pattern n); the answer is the pure-state amplitude and probability
    <n|psi> = lhaf(B_n, gamma_n) * <0|psi> / sqrt(prod n_i!),   p(n) = |<n|psi>|^2,
with B = A[:M, :M]^*, gamma = alpha - B alpha^* and
    <0|psi> = det(I - B B^*)^(1/4) * exp(-(|alpha|^2 - alpha^* . B alpha^*) / 2),
the conventions of thewalrus/quantum/fock_tensors.py:45-98 (pure_state_amplitude) with
det(Q)^(-1/4) written as det(I - B B^*)^(1/4) for a pure state.

Serving loop (``ProbabilityServer.serve``):
* requests arrive at their timestamps (Poisson streams in the benchmark);
* a batch is formed from the pending requests of one state as long as a stream slot is free and
  the batch's device memory fits the budget (admission by device memory).  With
  ``order="cost"`` (the default) pending requests are taken cheapest first -- the cost of a
  request is its sieve term count times (m + 1)^3 for its largest term matrix, known from the
  pattern before any work -- and a batch closes once its summed cost passes ``batch_cost``
  (about 25 ms of GPU work), so that small requests are not held back by a large one in the
  same plan (a plan answers all its members when its last term is done); ``order="arrival"``
  takes them oldest first with no cost limit;
* each batch is a plan whose loop-hafnian matrices are formed on the device from the resident
  state (gather kernel), executed on its own CUDA stream with stream-ordered memory, so batches
  admitted while others run overlap on the GPU;
* completed batches are read back as soon as their event fires and their memory is released.
Per request the server records arrival, completion and latency; ``summary`` gives p50/p99
latency and hafnians/s.
"""
import math
import time

import numpy as np

from . import _native as nat
from ._hafnian import matched_reps
from .workloads import haar_unitary

__all__ = ["GaussianState", "ProbabilityServer", "poisson_requests", "summary"]


class GaussianState:
    """Pure Gaussian state on M modes given by B (complex symmetric, ||B|| < 1) and alpha."""

    def __init__(self, B, alpha):
        self.B = np.ascontiguousarray(B, dtype=np.complex128)
        self.alpha = np.ascontiguousarray(alpha, dtype=np.complex128)
        self.M = self.B.shape[0]
        self.gamma = self.alpha - self.B @ self.alpha.conj()
        _, logdet = np.linalg.slogdet(np.eye(self.M) - self.B @ self.B.conj())
        quad = np.vdot(self.alpha, self.alpha).real - self.alpha.conj() @ self.B @ self.alpha.conj()
        self.vacuum = np.exp(0.25 * logdet) * np.exp(-0.5 * quad)
        self.device = None

    @classmethod
    def from_cov(cls, mu, cov, hbar=2):
        """State from its xp-quadrature means and covariance (pure states only): the Husimi
        matrix Q, A = X (I - Q^-1)^*, B = A[:M, :M]^* and alpha as in
        thewalrus/quantum/conversions.py:70-170, with <0|psi> = exp(-(|alpha|^2 -
        alpha^* B alpha^*)/2) / det(Q)^(1/4)."""
        mu = np.asarray(mu, dtype=np.float64)
        cov = np.asarray(cov, dtype=np.float64)
        M = len(cov) // 2
        eye = np.identity(M)
        x, xp, p = cov[:M, :M] * 2 / hbar, cov[:M, M:] * 2 / hbar, cov[M:, M:] * 2 / hbar
        adag_a = (x + p + 1j * (xp - xp.T) - 2 * eye) / 4
        a_a = (x - p + 1j * (xp + xp.T)) / 4
        Q = np.block([[adag_a, a_a.conj()], [a_a, adag_a.conj()]]) + np.identity(2 * M)
        W = (np.identity(2 * M) - np.linalg.inv(Q)).conj()
        B = W[M:, :M].conj()  # (X W)[:M, :M] = W[M:, :M]
        alpha = (mu[:M] + 1j * mu[M:]) / np.sqrt(2 * hbar)
        obj = cls(B, alpha)
        quad = np.vdot(alpha, alpha).real - alpha.conj() @ B @ alpha.conj()
        obj.vacuum = np.exp(-0.5 * quad) / np.sqrt(np.sqrt(np.linalg.det(Q)))
        return obj

    @classmethod
    def from_cov_on_device(cls, mu, cov, hbar=2):
        """``from_cov`` with the conversions on the GPU: the Husimi matrix, its Cholesky factor,
        the columns of Q^-1 that B needs, gamma and the vacuum amplitude are formed by one kernel
        from the covariance (``wg_state_create_from_cov``), and the state stays resident for the
        serving plans; B and gamma come back to the host only as copies."""
        dev, vacuum, B, gamma = nat.DeviceState.from_cov(cov, mu, hbar)
        obj = cls.__new__(cls)
        obj.B, obj.gamma, obj.M = B, gamma, B.shape[0]
        obj.alpha = (np.asarray(mu[:obj.M]) + 1j * np.asarray(mu[obj.M:])) / np.sqrt(2 * hbar)
        obj.vacuum = vacuum
        obj.device = dev
        return obj

    @classmethod
    def synthetic(cls, modes=64, seed=0, r_range=(0.3, 0.8), disp_var=0.1):
        """Haar interferometer U, squeezing r_i ~ U(r_range), B = U diag(tanh r) U^T,
        displacement alpha_i ~ CN(0, disp_var)."""
        rng = np.random.default_rng(seed)
        U = haar_unitary(modes, rng)
        r = rng.uniform(*r_range, size=modes)
        B = U @ np.diag(np.tanh(r)) @ U.T
        alpha = (rng.normal(size=modes) + 1j * rng.normal(size=modes)) * np.sqrt(disp_var / 2)
        return cls(B, alpha)

    def to_device(self):
        if self.device is None:
            self.device = nat.DeviceState(self.B, self.gamma)
        return self.device

    def norm(self, pattern):
        """<0|psi> / sqrt(prod n_i!) for the pattern."""
        return self.vacuum / math.sqrt(float(np.prod([math.factorial(int(k)) for k in pattern])))

    def trivial_loop_hafnian(self, pattern):
        """The loop hafnian for patterns with at most one photon (no sieve needed), else None."""
        N = int(np.sum(pattern))
        if N == 0:
            return 1.0 + 0j
        if N == 1:
            return complex(self.gamma[int(np.nonzero(np.asarray(pattern))[0][0])])
        return None


def poisson_requests(states, rate, count, photons=(8, 44), seed=0, max_rep=2):
    """``count`` requests with exponential inter-arrival times at ``rate`` per second; each picks a
    state uniformly and a pattern with an even total drawn uniformly from ``photons``."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    lo, hi = photons
    totals = [N for N in range(lo, hi + 1) if N % 2 == 0]
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        s = int(rng.integers(len(states)))
        M = states[s].M
        N = int(totals[rng.integers(len(totals))])
        pat = np.zeros(M, dtype=np.int64)
        placed = 0
        while placed < N:
            i = rng.integers(M)
            if pat[i] < max_rep:
                pat[i] += 1
                placed += 1
        out.append((t, s, pat))
    return out


class ProbabilityServer:
    """Continuous batching of probability requests over CUDA streams (see module docstring)."""

    def __init__(self, states, precision="fp64", max_batch=128, streams=3, mem_budget=None, chunk_scale=1.0,
                 order="cost", batch_cost=4e9):
        import torch

        self.torch = torch
        self.states = list(states)
        for s in self.states:
            s.to_device()
        self.precision = precision
        self.max_batch = int(max_batch)
        self.chunk_scale = chunk_scale
        self.streams = [torch.cuda.Stream() for _ in range(streams)]
        if mem_budget is None:
            free, _ = torch.cuda.mem_get_info()
            mem_budget = int(0.25 * free)
        self.mem_budget = int(mem_budget)
        if order not in ("cost", "arrival"):
            raise ValueError("order must be 'cost' or 'arrival'")
        self.order = order
        self.batch_cost = float(batch_cost)

    @staticmethod
    def request_cost(triple):
        """Relative GPU work of a request from its pairing (x, edge_reps, oddmode): sieve terms
        (loop kind: the first radix halved unless there is an unpaired mode) times (m + 1)^3 for
        the largest bordered term matrix, m = 2 * (edges with a nonzero repetition)."""
        _, reps, odd = triple
        reps = [int(r) for r in reps]
        if not reps:
            return 0.0
        steps = float((reps[0] + 2) // 2 if odd is None else reps[0] + 1)
        for r in reps[1:]:
            steps *= r + 1
        m = 2 * sum(1 for r in reps if r > 0)
        return steps * float(m + 2) ** 3

    @staticmethod
    def estimate_bytes(N):
        """Upper estimate of one request's plan memory (pool + partials + bookkeeping)."""
        n = N + (N % 2)
        return (n + 3) * (n + 1) * 16 + 8192 * 16 + 2048

    def serve(self, requests, time_scale=1.0, timeout=600.0):
        """Serve ``requests`` = [(arrival_s, state_index, pattern)] (sorted by arrival) in real time.

        Returns one dict per request: amplitude, probability, arrival, done, latency (seconds),
        batch id.
        """
        torch = self.torch
        R = len(requests)
        results = [None] * R
        pending = []  # waiting requests (indices), non-trivial ones only
        info = {}  # request -> (cost, pairing, photons)
        inflight = []
        free = list(range(len(self.streams)))
        mem_used = 0
        nxt = 0
        batch_id = 0
        done = 0
        t0 = time.perf_counter()
        while done < R:
            now = time.perf_counter() - t0
            if now > timeout:
                raise TimeoutError("serving did not finish within %.0f s" % timeout)
            progressed = False
            while nxt < R and requests[nxt][0] * time_scale <= now:
                j = nxt
                nxt += 1
                progressed = True
                _, sidx, pat = requests[j]
                triv = self.states[sidx].trivial_loop_hafnian(pat)
                if triv is not None:  # no photons or one: answered without the sieve
                    self._finish(results, requests, j, triv, time.perf_counter() - t0, -1, time_scale)
                    done += 1
                    continue
                triple = matched_reps(pat)
                info[j] = (self.request_cost(triple), triple, int(np.sum(pat)))
                pending.append(j)
            # completions
            for fl in list(inflight):
                if fl["event"].query():
                    vals = fl["plan"].read(fl["stream"].cuda_stream)
                    tdone = time.perf_counter() - t0
                    for j, v in zip(fl["reqs"], vals):
                        self._finish(results, requests, j, complex(v), tdone, fl["id"], time_scale)
                    done += len(fl["reqs"])
                    fl["plan"].close()
                    mem_used -= fl["bytes"]
                    free.append(fl["slot"])
                    inflight.remove(fl)
                    progressed = True
            # admission of a new batch: one state; cheapest (or oldest) first, within the cost
            # budget, the slots and the device memory
            if free and pending:
                if self.order == "cost":
                    pending.sort(key=lambda j: (info[j][0], j))
                sidx = requests[pending[0]][1]
                batch, est, work = [], 0, 0.0
                keep = []
                closed = False
                for j in pending:
                    if closed or len(batch) >= self.max_batch or requests[j][1] != sidx:
                        keep.append(j)
                        continue
                    cost, _, photons = info[j]
                    e = self.estimate_bytes(photons)
                    over_mem = batch and mem_used + est + e > self.mem_budget
                    over_cost = batch and self.order == "cost" and work + cost > self.batch_cost
                    if over_mem or over_cost:
                        keep.append(j)
                        closed = True
                        continue
                    batch.append(j)
                    est += e
                    work += cost
                pending = keep
                if batch:
                    slot = free.pop()
                    stream = self.streams[slot]
                    triples = [info[j][1] for j in batch]
                    plan = nat.Plan.from_requests(self.states[sidx].device, triples, self.precision,
                                                  chunk_scale=self.chunk_scale, stream=stream.cuda_stream)
                    plan.execute(stream.cuda_stream)
                    ev = torch.cuda.Event()
                    ev.record(stream)
                    nbytes = plan.device_bytes()
                    mem_used += nbytes
                    inflight.append({"plan": plan, "event": ev, "reqs": batch, "slot": slot, "stream": stream,
                                     "bytes": nbytes, "id": batch_id})
                    batch_id += 1
                    progressed = True
            if not progressed:
                time.sleep(20e-6)
        return results

    def _finish(self, results, requests, j, lhaf, tdone, bid, time_scale):
        arr, sidx, pat = requests[j]
        arr = arr * time_scale
        amp = lhaf * self.states[sidx].norm(pat)
        results[j] = {"amplitude": amp, "probability": abs(amp) ** 2, "arrival": arr, "done": tdone,
                      "latency": tdone - arr, "batch": bid, "photons": int(np.sum(pat))}


def summary(results, makespan=None):
    """p50/p99 latency (seconds) and hafnians/s of a served run."""
    lat = np.array([r["latency"] for r in results])
    span = makespan if makespan is not None else max(r["done"] for r in results) - min(r["arrival"] for r in results)
    return {"requests": len(results), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "hafnians_per_s": len(results) / span if span > 0 else float("inf"),
            "batches": len({r["batch"] for r in results if r["batch"] >= 0})}
