#!/usr/bin/env python
"""Chain-steps per second of SGLD(+RMSprop) on Bayesian logistic regression.

Workload (one "step" = one SGLD step of every chain): N = 1,000,000
observations, d = 256 fp32 features ~ N(0,1), labels Bernoulli(sigmoid(X w*))
with w* ~ N(0, 1/d), Gaussian prior N(0, I), 256 independent chains, minibatch
1024 per chain, step size 1e-3 -> 1e-5 (gamma 0.33) over 5,000 steps, RMSprop
(alpha 0.9, lambda 1e-5), minibatch indices from the numpy PCG64 streams of
NumpyDataLoader (seed = chain id), data from default_rng(20261203 + 2).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbsgmc|reference]

The default arm times K steps of the fused, graph-captured plan with the data
resident in HBM (``value``), the same run end to end through alias.sgld with
host buffers (``e2e``), the fused step kernel alone against the HBM roofline,
the plain one-chain unfused GPU form, and the CPU oracle on a bounded sample.
``--impl reference`` times the reference algorithm's CPU restatement on all
host cores.  One JSON line on rank 0.
"""

import argparse
import json
import math
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "jax-sgmc_gb300", ROOT):
  if str(_p) not in sys.path:
    sys.path.insert(0, str(_p))

N_OBS, D, CHAINS, MB = 1_000_000, 256, 256, 1024
K_CONFIG = 5000
FIRST, LAST, GAMMA = 1e-3, 1e-5, 0.33
METRIC = "chain-steps/sec at fixed posterior-moment error; fused vs plain, same GB300"
WORKLOAD = ("Bayesian logistic regression, SGLD+RMSprop: N=1,000,000, d=256 fp32, "
            "256 chains, minibatch 1024, 5,000-step polynomial schedule 1e-3->1e-5")
BYTES_PER_CHAIN_STEP = MB * (4 * D + 4)     # gathered fp32 rows + labels


def make_data():
  rng = np.random.default_rng(20261203 + 2)
  X = rng.standard_normal((N_OBS, D), dtype=np.float32)
  w_star = rng.normal(size=D) / math.sqrt(D)
  p = 1.0 / (1.0 + np.exp(-(X @ w_star.astype(np.float32))))
  y = (rng.random(N_OBS) < p).astype(np.float32)
  return X, y


def step_tables(total):
  from gbsgmc import scheduler
  its = max(total, K_CONFIG)
  ss = scheduler.polynomial_step_size_first_last(FIRST, LAST, GAMMA)
  bi = scheduler.initial_burn_in(0)
  th = scheduler.random_thinning(ss, bi, selections=min(1000, its))
  sch = scheduler.init_scheduler(step_size=ss, burn_in=bi, thinning=th)
  return scheduler.tables(sch, its)


def pcg_words(seed):
  """Device PCG64 words of the index stream of chain `seed`, as the
  NumpyDataLoader registers it."""
  from gbsgmc.data.numpy_loader import pcg64_words
  return pcg64_words(seed)


def shard_chains(rank, per_rank):
  """Weak scaling: rank r runs its own `per_rank` chains, ids
  [r * per_rank, (r + 1) * per_rank).  A chain's index stream is seeded with
  its id and its noise keyed by it, so a chain's samples do not depend on
  how chains are spread over ranks.  Returns (first id, ids)."""
  base = rank * per_rank
  return base, list(range(base, base + per_rank))


def max_over_ranks(value, world, device):
  """The slowest rank's time (all-reduce MAX); `value` itself for one rank."""
  if world <= 1:
    return value
  import torch
  import torch.distributed as dist
  t = torch.tensor([float(value)], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def dist_env():
  rank = int(os.environ.get("RANK", "0"))
  world = int(os.environ.get("WORLD_SIZE", "1"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  return rank, world, local


class Clocks:
  """Samples nvidia-smi clocks and throttle reasons during the timed region.
  start() returns once the sampler has printed its first line, so that the
  timed work that follows is inside its sampling window."""
  QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, gpu_index):
    self.gpu = gpu_index
    self.proc = None
    self.lines = []
    self.reader = None

  def start(self, wait_s=5.0):
    import threading
    try:
      self.proc = subprocess.Popen(
          ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
           "--format=csv,noheader,nounits", "-lms", "100"],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except (OSError, ValueError):
      self.proc = None
      return
    first = threading.Event()

    def read():
      for line in self.proc.stdout:
        self.lines.append(line)
        first.set()
      first.set()

    self.reader = threading.Thread(target=read, daemon=True)
    self.reader.start()
    first.wait(wait_s)

  def stop(self):
    if self.proc is None:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    self.proc.terminate()
    try:
      self.proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
      self.proc.kill()
      self.proc.wait()
    if self.reader is not None:
      self.reader.join(timeout=5)
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in self.lines:
      f = [x.strip() for x in line.split(",")]
      if len(f) < 9:
        continue
      try:
        sm.append(float(f[1]))
        smax.append(float(f[2]))
      except ValueError:
        continue
      for name, val in zip(names, f[5:9]):
        if val.lower().startswith("active"):
          reasons.add(name)
    if not sm:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax),
            "reasons": sorted(reasons), "samples": len(sm)}


def timed_repeats(run_region, barrier, min_seconds=2.0, min_repeats=3,
                  max_repeats=100000):
  """Times the same K-step region (``run_region(r)`` enqueues exactly K
  steps, repeat r) again and again with CUDA events on the current stream,
  each repeat bracketed by a barrier and a device synchronize, until
  ``min_seconds`` of wall time and ``min_repeats`` repeats have passed.
  Returns the per-repeat milliseconds."""
  import torch
  ms = []
  t0 = time.perf_counter()
  r = 0
  while r < max_repeats and (r < min_repeats or time.perf_counter() - t0 < min_seconds):
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    barrier()
    start.record()
    run_region(r)
    end.record()
    barrier()
    ms.append(start.elapsed_time(end))
    r += 1
  return ms


def measured_peak_hbm():
  p = ROOT / "MEASURED_PEAKS.json"
  if p.exists():
    try:
      return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except (KeyError, ValueError):
      pass
  return 6800.0, "fallback"


def profiled_traffic():
  """DRAM bytes of one fused SGLD step of all chains, from the committed ncu
  summary (dram__bytes_read.sum + dram__bytes_write.sum)."""
  p = ROOT / "profiles" / "glm_sgld_step_logistic_256x1024x256.md"
  if not p.exists():
    return None
  for line in p.read_text().splitlines():
    if line.startswith("traffic_bytes_per_step:"):
      try:
        return float(line.split(":", 1)[1].strip().split()[0])
      except ValueError:
        return None
  return None


# ---------------------------------------------------------------------------
# Posterior-moment error: Bayesian linear regression with a closed-form
# posterior (N = 10,000, d = 32, sigma 0.5, prior N(0, 10^2 I), minibatch
# 128, SGLD with RMSprop through alias.sgld).
# ---------------------------------------------------------------------------
CFG1_N, CFG1_D, CFG1_MB = 10_000, 32, 128
# Three alias.sgld calls, each starting from the previous call's last
# sample: (first step size, last step size, iterations, burn-in, kept).  The
# first call travels from w = 0 to the posterior (RMSprop moves each weight
# about one step size per step far from it), the second brings the chains'
# spread close to the posterior's, the third samples.  RMSprop alpha 0.999:
# the rms_prop adaption updates v with the current gradient before scaling
# that gradient by 1 / sqrt(v) (adaption.py:254-291), which widens the
# stationary distribution by about (1 - alpha) relative in variance, 11 %
# at the default alpha 0.9.
CFG1_PHASES = ((2e-3, 1e-3, 10_000, 9_999, 1),
               (1e-4, 5e-5, 10_000, 9_999, 1),
               (5e-6, 4e-6, 60_000, 36_000, 50))
CFG1_ALPHA = 0.999


def config1_data():
  rng = np.random.default_rng(20261203 + 1)
  X = rng.standard_normal((CFG1_N, CFG1_D), dtype=np.float32)
  w_star = rng.normal(size=CFG1_D)
  y = (X @ w_star + 0.5 * rng.normal(size=CFG1_N)).astype(np.float32)
  return X, y


def linear_posterior(X, y, sigma=0.5, prior_scale=10.0):
  """Closed-form Gaussian posterior (FP64): mean and covariance."""
  Xd = X.astype(np.float64)
  prec = Xd.T @ Xd / sigma ** 2 + np.eye(X.shape[1]) / prior_scale ** 2
  cov = np.linalg.inv(prec)
  return cov @ (Xd.T @ y.astype(np.float64)) / sigma ** 2, cov


def config1_moment_error(chains=16384):
  """Runs the config-1 chains through alias.sgld (CFG1_PHASES) and returns
  the relative errors of the kept samples' mean and per-weight variance
  against the closed-form posterior, with the chain-steps and seconds of
  the three calls."""
  import torch
  from gbsgmc import alias, data, likelihoods as L, potential
  X, y = config1_data()
  mu, cov = linear_posterior(X, y)
  loader = data.NumpyDataLoader(x=X, y=y)
  pot = potential.minibatch_potential(L.GaussianPrior(10.0),
                                      L.LinearGaussian(sigma=0.5), strategy="vmap")
  starts = [{"w": np.zeros(CFG1_D, np.float32)} for _ in range(chains)]
  steps = 0
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  for first, last, its, burn, kept in CFG1_PHASES:
    run = alias.sgld(pot, loader, cache_size=512, batch_size=CFG1_MB,
                     first_step_size=first, last_step_size=last, burn_in=burn,
                     accepted_samples=kept, rms_prop=True, alpha=CFG1_ALPHA)
    res = run(*starts, iterations=its)
    steps += chains * its
    W = np.stack([r["samples"]["variables"]["w"] for r in res], 1)  # [S, C, d]
    starts = [{"w": W[-1, c]} for c in range(chains)]
  seconds = time.perf_counter() - t0
  flat = W.reshape(-1, CFG1_D).astype(np.float64)
  var = np.diag(cov)
  return {"mean": float(np.linalg.norm(flat.mean(0) - mu) / np.linalg.norm(mu)),
          "var": float(np.linalg.norm(flat.var(0) - var) / np.linalg.norm(var)),
          "chains": chains, "chain_steps": steps, "seconds": seconds}


# ---------------------------------------------------------------------------
# CPU arms (oracle)
# ---------------------------------------------------------------------------

def cpu_chain_steps(X, y, chains, steps, threads):
  """Times ``steps`` SGLD steps of ``chains`` chains of the reference
  algorithm restated on the CPU (oracle); returns chain-steps/s."""
  from oracle import sgmc_oracle as O
  rngs = [O.loader_rng(c) for c in range(chains)]
  W = np.zeros((chains, D), np.float32)
  V = np.ones((chains, D), np.float32)
  h = np.full(steps, FIRST, np.float32)
  T = np.ones(steps, np.float32)
  t0 = time.perf_counter()
  O.sgld_glm_cpu_steps(X, y, W, V, rngs, (steps, MB), h, T, O.LOGISTIC,
                       prior_scale=1.0, threads=threads)
  dt = time.perf_counter() - t0
  return chains * steps / dt, dt


def run_reference(args):
  rank, world, _ = dist_env()
  if rank != 0:
    return
  threads = os.cpu_count() or 1
  X, y = make_data()
  # Size the per-step sample so that warmup + steps end within ~2 minutes.
  probe, dt = cpu_chain_steps(X, y, threads, 1, threads)
  per_step = max(1, min(CHAINS, int(probe * 110.0 / max(args.steps + args.warmup, 1))))
  cpu_chain_steps(X, y, per_step, max(args.warmup, 1), threads)
  value, dt = cpu_chain_steps(X, y, per_step, args.steps, threads)
  sample = f"{per_step} chains x {args.steps} steps of the {CHAINS}-chain workload"
  line = {
      "impl": "reference", "metric": METRIC, "value": value,
      "unit": "chain-steps/s", "n_gpus": args.gpus, "steps": args.steps,
      "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
      "dtype": "f32", "data": "synthetic (numpy default_rng(20261205))",
      "config": {"workload": WORKLOAD, "n_obs": N_OBS, "d": D, "chains": CHAINS,
                 "minibatch": MB, "sample": sample},
      "cpu_baseline": {"value": value, "unit": "chain-steps/s", "cores": threads,
                       "kind": "port", "sample": sample},
      "e2e": {"value": value, "unit": "chain-steps/s", "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": 0},
  }
  print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class Setup:
  """Data resident in HBM, the potential, and the chains of this rank."""

  def __init__(self, rank):
    import torch
    from gbsgmc import _build, _lib, data, likelihoods as L, potential
    _build.build()
    self.lib = _lib.load()
    self.X, self.y = make_data()
    self.loader = data.NumpyDataLoader(x=self.X, y=self.y)
    self.ds = self.loader.device_dataset()
    self.pot = potential.minibatch_potential(L.GaussianPrior(1.0), L.Logistic(),
                                             strategy="vmap")
    self.chain_base, _ = shard_chains(rank, CHAINS)
    self.W = torch.zeros((CHAINS, D), dtype=torch.float32, device="cuda")
    self.V = torch.ones((CHAINS, D), dtype=torch.float32, device="cuda")

  def plan(self, total):
    import torch
    from gbsgmc import engine
    h, T, keep, n_kept, _ = step_tables(total)
    words = np.array([pcg_words(self.chain_base + c) for c in range(CHAINS)],
                     np.uint64).view(np.int64)
    self.pcg = torch.from_numpy(words.copy()).cuda()
    self.tabs = [torch.from_numpy(a).cuda() for a in (h, T, keep)]
    return engine.SgldGlmPlan(
        self.pot, self.ds, self.W, self.V, 0.9, 1e-5, MB, *self.tabs, n_kept,
        engine.IndexSource(pcg=self.pcg, chain_base=self.chain_base),
        noise_seed=0, chain_base=self.chain_base, block_steps=50)


class FusedLauncher:
  """Direct launches of the fused step kernel on torch's current stream:
  one step per launch, or (multi=True, the plan's choice when its blocks run
  in one launch) eight steps per launch over the eight index sets."""

  def __init__(self, s, multi=False):
    import torch
    from gbsgmc import _lib
    self._lib = _lib
    self.ws = s.pot.workspace(CHAINS, MB, D)
    self.status = torch.zeros(1, dtype=torch.int32, device="cuda")
    self.idx = torch.empty((8, CHAINS, MB), dtype=torch.int32, device="cuda")
    self.stream = _lib.stream_handle()
    _lib.call("gbsgmc_index_draw_philox", 99, 0, CHAINS, 0, 8, MB, N_OBS,
              _lib.ptr(self.idx), MB, CHAINS * MB, self.stream)
    self.model, self._keep = s.pot.model(s.ds)
    self.W, self.V = s.W.clone(), s.V.clone()
    self.sched = _lib.sched(step_size=1e-5, temperature=1.0, offset=0)
    self.noise = _lib.noise(seed=5)
    self.steps_per_launch = 8 if multi else 1

  def __call__(self, i):
    L = self._lib
    if self.steps_per_launch > 1:
      L.call("gbsgmc_sgld_glm_steps", self.model, CHAINS, MB, L.ptr(self.idx),
             MB, CHAINS * MB, self.steps_per_launch, L.ptr(self.W),
             L.ptr(self.V), 0.9, 1e-5, self.sched, self.noise, None, None, None,
             None, L.ptr(self.ws), self.ws.numel(), L.ptr(self.status),
             self.stream)
      return
    L.call("gbsgmc_sgld_glm_step", self.model, CHAINS, MB, L.ptr(self.idx[i % 8]),
           MB, L.ptr(self.W), L.ptr(self.V), 0.9, 1e-5, self.sched, self.noise,
           None, None, None, None, L.ptr(self.ws), self.ws.numel(),
           L.ptr(self.status), self.stream)


def kernel_only(args):
  """A short run for profilers: three plan steps, ten more, then five direct
  launches of the fused step kernel (eight steps each when the plan runs a
  block of steps per launch)."""
  import torch
  rank, _, local = dist_env()
  torch.cuda.set_device(local)
  s = Setup(rank)
  plan = s.plan(args.warmup + 10)
  plan.run(0, args.warmup)
  plan.run(args.warmup, 10)
  torch.cuda.synchronize()
  plan.check_status()
  multi = plan.launch_shape()[5] > 1
  plan.close()
  f = FusedLauncher(s, multi=multi)
  for i in range(5):
    f(i)
  torch.cuda.synchronize()
  assert int(f.status.item()) == 0


def run_gbsgmc(args):
  import torch
  import torch.distributed as dist
  from gbsgmc import _lib, alias
  rank, world, local = dist_env()
  torch.cuda.set_device(local)
  if world > 1:
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))

  def barrier():
    if world > 1:
      dist.barrier()
    torch.cuda.synchronize()

  s = Setup(rank)
  K = args.steps
  # The schedule tables span the workload's 5,000 steps (or W + K if longer).
  total = max(args.warmup + K, K_CONFIG)
  plan = s.plan(total)
  span = total - args.warmup - K

  # W untimed warm-up steps, then the same K-step region timed again and
  # again (each repeat exactly K steps between barriers and device
  # synchronisation, CUDA events on the plan's stream order) for at least
  # 2 s, so that the clock sampler sees the load; the median repeat counts.
  plan.run(0, args.warmup)
  barrier()
  clocks = Clocks(local)
  clocks.start()
  region_ms = timed_repeats(
      lambda r: plan.run(args.warmup + ((r * K) % (span + 1) if span > 0 else 0), K),
      barrier, min_seconds=2.0)
  clk = clocks.stop()
  ms = float(np.median(region_ms))
  plan.check_status()
  ms = max_over_ranks(ms, world, "cuda")
  value = world * CHAINS * K / (ms / 1e3)
  launches = plan.launches(args.steps)
  shape = plan.launch_shape()
  finite = bool(torch.isfinite(s.W).all().item())
  plan.close()

  # The fused step kernel alone: average launch time on its stream.
  f = FusedLauncher(s, multi=shape[5] > 1)
  for i in range(5):
    f(i)
  reps = 200 if f.steps_per_launch == 1 else 25
  torch.cuda.synchronize()
  k0 = torch.cuda.Event(enable_timing=True)
  k1 = torch.cuda.Event(enable_timing=True)
  k0.record()
  for i in range(reps):
    f(i)
  k1.record()
  torch.cuda.synchronize()
  kernel_ms = k0.elapsed_time(k1) / reps
  bytes_per_launch = CHAINS * BYTES_PER_CHAIN_STEP * f.steps_per_launch
  achieved = bytes_per_launch / (kernel_ms / 1e3) / 1e9
  peak, peak_kind = measured_peak_hbm()

  # Plain one-chain unfused GPU form (8 launches per step).
  plain_steps = 300
  buf = torch.zeros(int(s.lib.gbsgmc_plain_buffer_bytes(MB, D)),
                    dtype=torch.uint8, device="cuda")
  w1 = torch.zeros((1, D), dtype=torch.float32, device="cuda")
  v1 = torch.ones((1, D), dtype=torch.float32, device="cuda")
  U1 = torch.zeros(1, dtype=torch.float64, device="cuda")

  def plain_step(k):
    _lib.call("gbsgmc_plain_sgld_glm_step", f.model, MB, _lib.ptr(f.idx[k % 8, 0]),
              _lib.ptr(w1), _lib.ptr(v1), 0.9, 1e-5,
              _lib.sched(step_size=1e-5, temperature=1.0, offset=k), f.noise,
              _lib.ptr(U1), _lib.ptr(buf), _lib.ptr(f.status), f.stream)

  for k in range(10):
    plain_step(k)
  torch.cuda.synchronize()
  p0 = time.perf_counter()
  for k in range(plain_steps):
    plain_step(k)
  torch.cuda.synchronize()
  plain_value = plain_steps / (time.perf_counter() - p0)

  # End to end through the public API: alias.sgld with host samples in and
  # numpy samples out; the dataset stays resident in HBM between calls.
  kw = dict(cache_size=512, batch_size=MB, first_step_size=FIRST,
            last_step_size=LAST, rms_prop=True)
  init = [{"w": np.zeros(D, np.float32)} for _ in range(CHAINS)]
  # Warm the path at the timed shape: the plan's autotuner runs once per
  # process and shape (chains, minibatch, features), like a first-call
  # compile, and later plans of that shape reuse its choice.
  alias.sgld(s.pot, s.loader, accepted_samples=1, **kw)(
      *init, iterations=args.warmup)
  e2e_run = alias.sgld(s.pot, s.loader, accepted_samples=min(1000, args.steps),
                       **kw)
  # Whole calls, each K steps from host samples to numpy samples, repeated
  # for at least 1 s; the median call counts.
  e2e_times = []
  t_all = time.perf_counter()
  while len(e2e_times) < 3 or time.perf_counter() - t_all < 1.0:
    barrier()
    e0 = time.perf_counter()
    results = e2e_run(*init, iterations=args.steps)
    barrier()
    e2e_times.append(time.perf_counter() - e0)
    if len(e2e_times) >= 200:
      break
  e2e_s = float(np.median(e2e_times))
  e2e_s = max_over_ranks(e2e_s, world, "cuda")
  kept = results[0]["sample_count"]
  h2d = CHAINS * (D * 4 + 40) + args.steps * 12
  d2h = CHAINS * kept * (D * 4 + 8)
  e2e_value = world * CHAINS * args.steps / e2e_s

  # Posterior-moment error of the same fused SGLD path on the workload
  # with a closed-form posterior (rank 0 only).
  moment = None
  if rank == 0:
    m = config1_moment_error()
    moment = {"mean": m["mean"], "var": m["var"], "bar": 0.02,
              "workload": ("Bayesian linear regression N=10,000, d=32, sigma 0.5, "
                           "prior N(0,10^2 I), minibatch 128, SGLD+RMSprop "
                           f"(alpha {CFG1_ALPHA}) via alias.sgld, "
                           f"{m['chains']} chains; steps/burn-in/kept per call "
                           + ", ".join(f"{i}/{b}/{k} at h {f:g}->{l:g}"
                                       for f, l, i, b, k in CFG1_PHASES)),
              "against": "closed-form Gaussian posterior (FP64): relative L2 "
                         "error of the mean and of the per-weight variances",
              "chain_steps_per_s": m["chain_steps"] / m["seconds"]}

  # The tensor-core workload in brief: OBABO on the tanh network (rank 0).
  mlp = mlp_record() if rank == 0 else None

  # CPU oracle on a bounded sample (rank 0 only).
  cpu = None
  if rank == 0:
    threads = os.cpu_count() or 1
    # A short probe sizes a sample of about 10 s: the workload's chains for
    # as many steps as that takes (2 to 200).  The probe's rate, with its
    # fixed costs, is about half the sustained one, hence 20 s of it.
    probe, _ = cpu_chain_steps(s.X, s.y, 2 * threads, 2, threads)
    cpu_steps = int(min(200, max(2, round(20.0 * probe / CHAINS))))
    val, cpu_dt = cpu_chain_steps(s.X, s.y, CHAINS, cpu_steps, threads)
    cpu = {"value": val, "unit": "chain-steps/s", "cores": threads,
           "kind": "port",
           "sample": f"{CHAINS} chains x {cpu_steps} steps, {cpu_dt:.1f} s "
                     f"(numpy restatement, {threads} threads)"}

  if rank == 0:
    line = {
        "metric": METRIC, "value": value, "unit": "chain-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (numpy default_rng(20261205); X 1.02 GB resident in HBM)",
        "config": {"workload": WORKLOAD, "n_obs": N_OBS, "d": D,
                   "chains_per_gpu": CHAINS, "minibatch": MB,
                   "index_stream": "numpy PCG64 per chain, bit-exact",
                   "noise": "Philox4x32-10",
                   "l2": "inputs larger than L2 (X 1.02 GB, random rows)",
                   "parallelism": f"chains sharded, {world} replica(s)",
                   "graph_block_steps": 50,
                   "timing": (f"median of {len(region_ms)} repeats of the K-step region "
                              f"(min {min(region_ms):.4f} ms, max {max(region_ms):.4f} ms); "
                              f"e2e: median of {len(e2e_times)} calls"),
                   "launch_shape": {"ctas_or_items_per_chain": shape[0],
                                    "rows_per_warp": shape[1],
                                    "warps_per_cta": shape[2],
                                    "prefetch_tiles": shape[3],
                                    "dynamic_items": shape[4],
                                    "steps_per_launch": shape[5],
                                    "chosen_by": "autotuner"}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (None if profiled_traffic() is None else
                                 profiled_traffic() * f.steps_per_launch),
                     "steps_per_launch": f.steps_per_launch,
                     "peak_kind": f"{peak_kind} hbm_gbs",
                     "kernel": "glm_kernel (fused SGLD step)",
                     "kernel_ms": kernel_ms,
                     "algorithmic_bytes_per_launch": bytes_per_launch},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "chain-steps/s",
                "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps,
                "api": "gbsgmc.alias.sgld(...)(*256 samples, iterations=K)"},
        "plain_gpu": {"value": plain_value, "unit": "chain-steps/s",
                      "form": "one chain, 8 unfused launches per step",
                      "fused_over_plain": value / world / plain_value},
        "moment_error": moment,
        "mlp_obabo": mlp,
        "clocks": clk, "finite": finite,
        "device_status": int(f.status.item()),
    }
    print(json.dumps(line), flush=True)
  if world > 1:
    dist.destroy_process_group()


# ---------------------------------------------------------------------------
# MLP regression workload: 64 chains of OBABO on the 64-1024-1024-1 tanh
# network (BF16 tcgen05 GEMMs), minibatch 2048 of N = 500,000.
# ---------------------------------------------------------------------------
MLP_N, MLP_D, MLP_H, MLP_CHAINS, MLP_MB = 500_000, 64, 1024, 64, 2048
MLP_PMATMUL = MLP_D * MLP_H + MLP_H * MLP_H + MLP_H
MLP_FLOP_PER_GRAD = 6 * MLP_MB * MLP_PMATMUL      # forward 2, adjoint 4
MLP_WORKLOAD = ("Bayesian MLP regression, OBABO: 64-1024-1024-1 tanh "
                "(1,117,185 params/chain), sigma=0.1, N=500,000, 64 chains, "
                "minibatch 2048, BF16 GEMMs with FP32 accumulation")


def mlp_data():
  """X ~ N(0,1) [N, 64], targets from a random teacher network + N(0, 0.1^2)."""
  from gbsgmc import likelihoods as L
  rng = np.random.default_rng(20261203 + 3)
  lik = L.MLPGaussian(d_in=MLP_D, h1=MLP_H, h2=MLP_H, sigma=0.1)
  X = rng.standard_normal((MLP_N, MLP_D), dtype=np.float32)
  teacher = lik.unravel(lik.init(rng).astype(np.float64))
  y = np.empty(MLP_N, np.float32)
  try:
    import torch
    gpu = torch.cuda.is_available()
  except ImportError:
    gpu = False
  if gpu:
    # The teacher's forward pass in FP64 on the GPU (about 1e12 flop).
    tw = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in teacher.items()}
  for a in range(0, MLP_N, 50_000):
    if gpu:
      xb = torch.from_numpy(X[a:a + 50_000]).cuda().double()
      z1 = torch.tanh(xb @ tw["W1"] + tw["b1"])
      z2 = torch.tanh(z1 @ tw["W2"] + tw["b2"])
      f = ((z2 @ tw["W3"])[:, 0] + tw["b3"][0]).cpu().numpy()
    else:
      xb = X[a:a + 50_000].astype(np.float64)
      z1 = np.tanh(xb @ teacher["W1"] + teacher["b1"])
      z2 = np.tanh(z1 @ teacher["W2"] + teacher["b2"])
      f = (z2 @ teacher["W3"])[:, 0] + teacher["b3"][0]
    y[a:a + 50_000] = f + 0.1 * rng.standard_normal(min(50_000, MLP_N - a))
  inits = np.stack([lik.init(np.random.default_rng(1000 + c))
                    for c in range(MLP_CHAINS)])
  return lik, X, y, inits


def mlp_cpu_grad_rate(lik, X, y, W, reps, threads):
  """Gradients/s of the float64 oracle on one chain (bounded sample)."""
  from oracle import sgmc_oracle as O
  os.environ.setdefault("OMP_NUM_THREADS", str(threads))
  rng = np.random.default_rng(5)
  t0 = time.perf_counter()
  for _ in range(reps):
    idx = rng.integers(0, MLP_N, size=(1, MLP_MB))
    O.mlp_potential(W[:1], X, y, idx, MLP_N, MLP_D, MLP_H, MLP_H, 0.1,
                    prior_scale=1.0)
  return reps / (time.perf_counter() - t0)


def run_mlp_reference(args):
  """The oracle on all host cores for the MLP workload (rank 0 only)."""
  rank, _, _ = dist_env()
  if rank != 0:
    return
  lik, X, y, inits = mlp_data()
  threads = os.cpu_count() or 1
  for _ in range(args.warmup):
    mlp_cpu_grad_rate(lik, X, y, inits, 1, threads)
  rate = mlp_cpu_grad_rate(lik, X, y, inits, max(1, args.steps // 50), threads) / 2.0
  print(json.dumps({
      "impl": "reference", "metric": METRIC, "value": rate, "unit": "chain-steps/s",
      "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
      "higher_is_better": True, "config": {"workload": MLP_WORKLOAD},
      "cpu_baseline": {"value": rate, "unit": "chain-steps/s", "cores": threads,
                       "kind": "port", "sample": "float64 oracle gradients of one chain"},
      "e2e": {"value": rate, "unit": "chain-steps/s", "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": 0}}), flush=True)


# ---------------------------------------------------------------------------
# reSGLD workload: 32 replicas of SGLD on the same network, temperatures
# 100^(r/31), minibatch sizes drawn uniformly from 64..4096, exchange
# attempts between adjacent replicas every 50 steps.
# ---------------------------------------------------------------------------
RE_REPLICAS, RE_EVERY = 32, 50
RE_WORKLOAD = ("reSGLD on the MLP regression model: 32 replicas at T_r = 100^(r/31), "
               "minibatch n_r ~ U{64..4096} per replica, adjacent exchange every "
               "50 steps (FP64 log-ratio), SGLD with RMSprop")


def resgld_sizes():
  return np.random.default_rng(20261203 + 4).integers(64, 4097, size=RE_REPLICAS)


def run_resgld(args):
  import torch
  from gbsgmc import engine, likelihoods as L, potential, data
  rank, world, local = dist_env()
  torch.cuda.set_device(local)
  lik, X, y, inits = mlp_data()
  ds = data.NumpyDataLoader(x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  rows = resgld_sizes().astype(np.int32)
  n_max = int((rows.max() + 127) // 128 * 128)
  ladder = (100.0 ** (np.arange(RE_REPLICAS) / (RE_REPLICAS - 1))).astype(np.float32)
  steps = max(RE_EVERY, args.steps // RE_EVERY * RE_EVERY)
  warm = RE_EVERY
  total = warm + steps
  h = torch.full((total,), 1e-5, dtype=torch.float32, device="cuda")
  t = torch.ones(total, dtype=torch.float32, device="cuda")
  Xd = torch.from_numpy(inits[:RE_REPLICAS].copy()).cuda()
  Vd = torch.ones_like(Xd)   # RMSprop preconditioner (alpha 0.9, lambda 1e-5)
  words = np.array([pcg_words(RE_REPLICAS * rank + c) for c in range(RE_REPLICAS)],
                   np.uint64).view(np.int64)
  pcg = torch.from_numpy(words.copy()).cuda()
  plan = engine.ResgldPlan(pot, ds, Xd, Vd, rows, n_max, ladder, h, t,
                           engine.IndexSource(pcg=pcg, chain_base=RE_REPLICAS * rank),
                           noise_seed=11, swap_seed=12, every=RE_EVERY)
  plan.run(0, warm)
  torch.cuda.synchronize()
  clocks = Clocks(local)
  clocks.start()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  plan.run(warm, steps)
  e1.record()
  torch.cuda.synchronize()
  clk = clocks.stop()
  ms = e0.elapsed_time(e1)
  plan.check_status()
  finite = bool(torch.isfinite(Xd).all().item())
  exchanges = int(plan.counts.sum().item())
  value = world * RE_REPLICAS * steps / (ms / 1e3)
  launches = plan.launches(steps)
  plan.close()
  # The ragged batched gradient alone.
  idx = torch.randint(0, MLP_N, (RE_REPLICAS, n_max), dtype=torch.int32, device="cuda")
  rows_d = torch.from_numpy(rows).cuda()
  for _ in range(3):
    pot.evaluate(Xd, idx, ds, grad=True, rows=rows_d)
  torch.cuda.synchronize()
  g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  g0.record()
  for _ in range(10):
    pot.evaluate(Xd, idx, ds, grad=True, rows=rows_d)
  g1.record()
  torch.cuda.synchronize()
  grad_ms = g0.elapsed_time(g1) / 10
  flops = 6.0 * float(rows.sum()) * MLP_PMATMUL
  peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
      if (ROOT / "MEASURED_PEAKS.json").exists() else {}
  peak = peaks.get("bf16_tflops_sustained", 1700.0)
  achieved = flops / (grad_ms / 1e3) / 1e12
  # End to end through the package: host replicas in, plan built, the steps
  # run, replicas and exchange counts back on the host.
  torch.cuda.synchronize()
  s0 = time.perf_counter()
  Xh = inits[:RE_REPLICAS].copy()
  X2 = torch.from_numpy(Xh).cuda()
  V2 = torch.ones_like(X2)
  pcg2 = torch.from_numpy(words.copy()).cuda()
  plan2 = engine.ResgldPlan(pot, ds, X2, V2, rows, n_max, ladder, h, t,
                            engine.IndexSource(pcg=pcg2, chain_base=RE_REPLICAS * rank),
                            noise_seed=11, swap_seed=12, every=RE_EVERY)
  plan2.run(0, steps)
  X_out = X2.cpu().numpy()
  counts_out = plan2.counts.cpu().numpy()
  plan2.check_status()
  plan2.close()
  e2e_s = time.perf_counter() - s0
  e2e_value = world * RE_REPLICAS * steps / e2e_s
  h2d = 2 * Xh.nbytes + words.nbytes
  d2h = X_out.nbytes + counts_out.nbytes
  cpu = None
  if rank == 0:
    threads = os.cpu_count() or 1
    grad_rate = mlp_cpu_grad_rate(lik, X, y, inits, 3, threads)
    # One replica-step is one gradient at n_r rows; the sample is at 2048.
    cpu_rate = grad_rate * MLP_MB / float(rows.mean())
    cpu = {"value": cpu_rate, "unit": "chain-steps/s", "cores": threads, "kind": "port",
           "sample": f"3 float64 gradients of one replica at n = {MLP_MB} (numpy oracle, "
                     f"{threads} threads), scaled to the mean minibatch {rows.mean():.0f}"}
  if rank == 0:
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "chain-steps/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 GEMMs, f32 state, f64 exchange",
        "data": "synthetic (teacher MLP targets, numpy default_rng(20261206))",
        "config": {"workload": RE_WORKLOAD, "replicas": RE_REPLICAS,
                   "minibatch_sizes": rows.tolist(), "sum_minibatch": int(rows.sum()),
                   "exchange_every": RE_EVERY, "exchanges_accepted": exchanges,
                   "graph_block_steps": 50},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": "measured bf16_tflops_sustained",
                     "kernel": "ragged batched value-and-gradient, 32 replicas",
                     "kernel_ms": grad_ms, "algorithmic_flop_per_launch": flops},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "chain-steps/s",
                "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
                "api": "gbsgmc.engine.ResgldPlan from host replicas, results to host"},
        "clocks": clk, "finite": finite}), flush=True)


# ---------------------------------------------------------------------------
# CNN workload: 8 chains of OBABO on the conv classifier, minibatch 256 of
# N = 50,000 synthetic 32x32x3 images.
# ---------------------------------------------------------------------------
CNN_N, CNN_CHAINS, CNN_MB = 50_000, 8, 256
CNN_MAC_PER_IMAGE = (32 * 32 * 32 * 27 + 16 * 16 * 64 * 288 + 8 * 8 * 128 * 576
                     + 2048 * 10)
CNN_FLOP_PER_GRAD = 6 * CNN_MB * CNN_MAC_PER_IMAGE   # 2 flop per MAC, 3 passes
CNN_WORKLOAD = ("Bayesian CNN classifier, OBABO: conv3x3 32/64/128 (ReLU, 2x2 "
                "max-pool, SAME) + dense 10, P=113,738; N=50,000 synthetic "
                "32x32x3 images, 10 classes; prior N(0,I); 8 chains, minibatch 256; "
                "convolutions as BF16 GEMMs")


def cnn_data():
  from gbsgmc import likelihoods as L
  rng = np.random.default_rng(20261203 + 5)
  images = rng.standard_normal((CNN_N, 32, 32, 3), dtype=np.float32)
  labels = rng.integers(0, 10, size=CNN_N).astype(np.float32)
  lik = L.CNNSoftmax()
  inits = np.stack([lik.init(np.random.default_rng(2000 + c)) for c in range(CNN_CHAINS)])
  return lik, images, labels, inits


def run_cnn(args):
  import torch
  from gbsgmc import alias, data, engine, likelihoods as L, potential
  rank, world, local = dist_env()
  torch.cuda.set_device(local)
  lik, images, labels, inits = cnn_data()
  loader = data.NumpyDataLoader(image=images, label=labels)
  ds = loader.device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  total = args.warmup + args.steps
  h = torch.full((total,), 1e-5, dtype=torch.float32, device="cuda")
  t = torch.ones(total, dtype=torch.float32, device="cuda")
  Xd = torch.from_numpy(inits).cuda()
  Pd = torch.zeros_like(Xd)
  words = np.array([pcg_words(CNN_CHAINS * rank + c) for c in range(CNN_CHAINS)],
                   np.uint64).view(np.int64)
  pcg = torch.from_numpy(words.copy()).cuda()
  plan = engine.NetPlan(pot, ds, Xd, Pd, CNN_MB, "obabo", h, t,
                        engine.IndexSource(pcg=pcg, chain_base=CNN_CHAINS * rank),
                        noise_seed=13, chain_base=CNN_CHAINS * rank, friction=1.0)
  plan.run(0, args.warmup)
  torch.cuda.synchronize()
  clocks = Clocks(local)
  clocks.start()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  plan.run(args.warmup, args.steps)
  e1.record()
  torch.cuda.synchronize()
  clk = clocks.stop()
  ms = e0.elapsed_time(e1)
  plan.check_status()
  finite = bool(torch.isfinite(Xd).all().item())
  value = world * CNN_CHAINS * args.steps / (ms / 1e3)
  launches = plan.launches(args.steps)
  plan.close()
  idx = torch.randint(0, CNN_N, (CNN_CHAINS, CNN_MB), dtype=torch.int32, device="cuda")
  for _ in range(3):
    pot.evaluate(Xd, idx, ds, grad=True)
  torch.cuda.synchronize()
  g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  g0.record()
  for _ in range(20):
    pot.evaluate(Xd, idx, ds, grad=True)
  g1.record()
  torch.cuda.synchronize()
  grad_ms = g0.elapsed_time(g1) / 20
  flops = CNN_CHAINS * CNN_FLOP_PER_GRAD
  peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
      if (ROOT / "MEASURED_PEAKS.json").exists() else {}
  peak = peaks.get("bf16_tflops_sustained", 1700.0)
  achieved = flops / (grad_ms / 1e3) / 1e12
  # Plain one-chain fp32 form: the same network in torch fp32 (cuDNN
  # convolutions) with autograd, one OBABO step per chain-step.
  F = torch.nn.functional
  imgs = torch.from_numpy(images).cuda()
  labs = torch.from_numpy(labels).cuda().long()
  from gbsgmc import likelihoods as L
  cnn_lik = L.CNNSoftmax()

  def plain_grad(w, rows):
    w = w.detach().requires_grad_(True)
    prm = cnn_lik.unravel(w)   # views of w in the sorted-key ravel order
    x = imgs[rows].permute(0, 3, 1, 2)
    for l in range(3):
      layer = prm[f"conv{l + 1}"]
      k = layer["w"].permute(3, 2, 0, 1)   # HWIO -> OIHW
      x = F.max_pool2d(F.relu(F.conv2d(x, k, layer["b"], padding=1)), 2)
    logits = x.permute(0, 2, 3, 1).reshape(CNN_MB, -1) @ prm["linear"]["w"] + \
        prm["linear"]["b"]
    U = (CNN_N / CNN_MB) * F.cross_entropy(logits, labs[rows], reduction="sum") + \
        0.5 * (w * w).sum()
    U.backward()
    return w.grad

  w1 = Xd[0].clone()
  p1 = torch.zeros_like(w1)

  def plain_step():
    nonlocal w1, p1
    hh, keep = 1e-5, math.exp(-1e-5)
    p1 = math.sqrt(keep) * p1 + math.sqrt(1 - keep) * torch.randn_like(p1)
    p1 = p1 - 0.5 * hh * plain_grad(w1, torch.randint(0, CNN_N, (CNN_MB,), device="cuda"))
    w1 = w1 + hh * p1
    p1 = p1 - 0.5 * hh * plain_grad(w1, torch.randint(0, CNN_N, (CNN_MB,), device="cuda"))
    p1 = math.sqrt(keep) * p1 + math.sqrt(1 - keep) * torch.randn_like(p1)

  for _ in range(3):
    plain_step()
  torch.cuda.synchronize()
  q0 = time.perf_counter()
  for _ in range(20):
    plain_step()
  torch.cuda.synchronize()
  plain_value = 20 / (time.perf_counter() - q0)
  # End to end through alias.obabo.
  kw = dict(cache_size=32, batch_size=CNN_MB, integration_steps=10, friction=1.0,
            first_step_size=1e-5, last_step_size=1e-6)
  trees = [lik.unravel(inits[c]) for c in range(CNN_CHAINS)]
  alias.obabo(pot, loader, accepted_samples=1, **kw)(*trees[:2], iterations=2)
  its = max(2, args.steps // 10)
  torch.cuda.synchronize()
  s0 = time.perf_counter()
  res = alias.obabo(pot, loader, accepted_samples=1, **kw)(*trees, iterations=its)
  torch.cuda.synchronize()
  e2e_value = CNN_CHAINS * its * 10 / (time.perf_counter() - s0)
  P = lik.param_count
  cpu = None
  if rank == 0:
    from oracle import sgmc_oracle as O   # the CPU baseline leg
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(5)
    t0 = time.perf_counter()
    for _ in range(2):
      O.cnn_potential(inits[0], images.reshape(CNN_N, -1), labels,
                      rng.integers(0, CNN_N, size=CNN_MB), CNN_N, prior_scale=1.0)
    rate = 2 / (time.perf_counter() - t0) / 2.0
    cpu = {"value": rate, "unit": "chain-steps/s", "cores": threads, "kind": "port",
           "sample": f"2 float64 gradients of one chain (numpy oracle, {threads} threads); "
                     "an OBABO step is two gradients"}
  if rank == 0:
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "chain-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 GEMMs, f32 state",
        "data": "synthetic (images ~N(0,1), labels U{0..9}, numpy default_rng(20261208)); "
                "614 MB resident in HBM",
        "config": {"workload": CNN_WORKLOAD, "chains_per_gpu": CNN_CHAINS,
                   "minibatch": CNN_MB, "integrator": "OBABO (2 gradients per step)",
                   "index_stream": "numpy PCG64 per chain, bit-exact",
                   "graph_block_steps": 50},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": "measured bf16_tflops_sustained",
                     "kernel": "batched value-and-gradient (8 tcgen05 GEMMs + im2col, "
                               "pooling, dense kernels), 8 chains",
                     "kernel_ms": grad_ms, "algorithmic_flop_per_launch": flops},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "chain-steps/s",
                "h2d_bytes_per_step": CNN_CHAINS * P * 4 / (its * 10),
                "d2h_bytes_per_step": CNN_CHAINS * res[0]["sample_count"] * (P * 4 + 8)
                / (its * 10),
                "api": "gbsgmc.alias.obabo(...)(*8 samples, iterations=K/10)"},
        "plain_gpu": {"value": plain_value, "unit": "chain-steps/s",
                      "form": "one chain, torch fp32 ops (cuDNN convolutions) + autograd",
                      "fused_over_plain": value / world / plain_value},
        "clocks": clk, "finite": finite}), flush=True)


def cnn_kernel_only(args):
  """`--steps` batched value-and-gradient calls of the 8-chain CNN workload
  and nothing else (for profilers); no JSON line."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  lik, images, labels, inits = cnn_data()
  ds = data.NumpyDataLoader(image=images, label=labels).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  W = torch.from_numpy(inits).cuda()
  idx = torch.randint(0, CNN_N, (CNN_CHAINS, CNN_MB), dtype=torch.int32, device="cuda")
  for _ in range(args.steps):
    pot.evaluate(W, idx, ds, grad=True)
  torch.cuda.synchronize()
  pot.check_status()


def mlp_kernel_only(args):
  """`--steps` batched value-and-gradient calls of the 64-chain workload,
  then `--steps` OBABO steps of the network plan (a short run for
  profilers); no JSON line."""
  import torch
  from gbsgmc import data, likelihoods as L, potential
  rng = np.random.default_rng(20261203 + 3)
  lik = L.MLPGaussian(d_in=MLP_D, h1=MLP_H, h2=MLP_H, sigma=0.1)
  X = rng.standard_normal((MLP_N, MLP_D), dtype=np.float32)
  y = rng.standard_normal(MLP_N).astype(np.float32)
  ds = data.NumpyDataLoader(x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  W = torch.from_numpy(np.stack([lik.init(rng) for _ in range(MLP_CHAINS)])).cuda()
  idx = torch.randint(0, MLP_N, (MLP_CHAINS, MLP_MB), dtype=torch.int32, device="cuda")
  for _ in range(args.steps):
    pot.evaluate(W, idx, ds, grad=True)
  torch.cuda.synchronize()
  pot.check_status()
  # Then `--steps` OBABO steps of the graph-captured plan (one block).
  from gbsgmc import engine
  words = np.array([pcg_words(c) for c in range(MLP_CHAINS)], np.uint64).view(np.int64)
  pcg = torch.from_numpy(words.copy()).cuda()
  h = torch.full((args.steps,), 1e-7, dtype=torch.float32, device="cuda")
  t = torch.ones(args.steps, dtype=torch.float32, device="cuda")
  plan = engine.NetPlan(pot, ds, W, torch.zeros_like(W), MLP_MB, "obabo", h, t,
                        engine.IndexSource(pcg=pcg), noise_seed=7, friction=1.0,
                        block_steps=args.steps)
  plan.run(0, args.steps)
  torch.cuda.synchronize()
  plan.check_status()
  plan.close()


def mlp_record(steps=20, warmup=3):
  """A compact record of the tanh-network workload for the default line:
  `steps` OBABO steps of its 64 chains (minibatch 2048, graph-captured
  network plan; two value-and-gradient calls per step) timed with CUDA
  events after `warmup` steps, and the batched value and gradient alone
  against the sustained BF16 peak."""
  import torch
  from gbsgmc import data, engine, likelihoods as L, potential
  lik, X, y, inits = mlp_data()
  ds = data.NumpyDataLoader(copy=False, x=X, y=y).device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  total = warmup + steps
  h = torch.full((total,), 1e-7, dtype=torch.float32, device="cuda")
  t = torch.ones(total, dtype=torch.float32, device="cuda")
  Xd = torch.from_numpy(inits).cuda()
  from gbsgmc.data.numpy_loader import pcg64_words_many
  pcg = torch.from_numpy(pcg64_words_many(range(MLP_CHAINS)).view(np.int64)).cuda()
  plan = engine.NetPlan(pot, ds, Xd, torch.zeros_like(Xd), MLP_MB, "obabo", h, t,
                        engine.IndexSource(pcg=pcg), noise_seed=7, friction=1.0)
  plan.run(0, warmup)
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record()
  plan.run(warmup, steps)
  e1.record()
  torch.cuda.synchronize()
  ms = e0.elapsed_time(e1) / steps
  plan.check_status()
  launches = plan.launches(steps)
  plan.close()
  idx = torch.randint(0, MLP_N, (MLP_CHAINS, MLP_MB), dtype=torch.int32, device="cuda")
  for _ in range(3):
    pot.evaluate(Xd, idx, ds, grad=True)
  torch.cuda.synchronize()
  g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  g0.record()
  for _ in range(10):
    pot.evaluate(Xd, idx, ds, grad=True)
  g1.record()
  torch.cuda.synchronize()
  pot.check_status()
  grad_ms = g0.elapsed_time(g1) / 10
  peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
      if (ROOT / "MEASURED_PEAKS.json").exists() else {}
  peak = peaks.get("bf16_tflops_sustained", 1700.0)
  kind = "measured bf16_tflops_sustained" if "bf16_tflops_sustained" in peaks else \
      "fallback"
  achieved = MLP_CHAINS * MLP_FLOP_PER_GRAD / (grad_ms / 1e3) / 1e12
  return {"workload": MLP_WORKLOAD, "value": MLP_CHAINS / (ms / 1e3),
          "unit": "chain-steps/s", "ms_per_step": ms, "steps": steps,
          "gpu_launches": launches, "dtype": "bf16 GEMMs, fp32 accumulation",
          "finite": bool(torch.isfinite(Xd).all().item()),
          "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                       "unit": "TFLOP/s", "frac": achieved / peak,
                       "peak_kind": kind,
                       "kernel": "batched value and gradient (5 tcgen05 GEMMs + "
                                 "epilogue kernels)",
                       "kernel_ms": grad_ms,
                       "algorithmic_flop_per_launch": MLP_CHAINS * MLP_FLOP_PER_GRAD}}


def run_mlp(args):
  import torch
  from gbsgmc import _lib, alias, data, engine, likelihoods as L, potential
  rank, world, local = dist_env()
  torch.cuda.set_device(local)
  lik, X, y, inits = mlp_data()
  loader = data.NumpyDataLoader(x=X, y=y)
  ds = loader.device_dataset()
  pot = potential.minibatch_potential(L.GaussianPrior(1.0), lik)
  total = args.warmup + args.steps
  h = torch.full((total,), 1e-7, dtype=torch.float32, device="cuda")
  t = torch.ones(total, dtype=torch.float32, device="cuda")
  Xd = torch.from_numpy(inits).cuda()
  Pd = torch.zeros_like(Xd)
  words = np.array([pcg_words(MLP_CHAINS * rank + c) for c in range(MLP_CHAINS)],
                   np.uint64).view(np.int64)
  pcg = torch.from_numpy(words.copy()).cuda()
  isrc = engine.IndexSource(pcg=pcg, chain_base=MLP_CHAINS * rank)
  plan = engine.NetPlan(pot, ds, Xd, Pd, MLP_MB, "obabo", h, t, isrc,
                        noise_seed=7, chain_base=MLP_CHAINS * rank, friction=1.0)
  plan.run(0, args.warmup)
  torch.cuda.synchronize()
  clocks = Clocks(local)
  clocks.start()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  torch.cuda.synchronize()
  e0.record()
  plan.run(args.warmup, args.steps)
  e1.record()
  torch.cuda.synchronize()
  clk = clocks.stop()
  ms = e0.elapsed_time(e1)
  plan.check_status()
  finite = bool(torch.isfinite(Xd).all().item())
  value = world * MLP_CHAINS * args.steps / (ms / 1e3)
  launches = plan.launches(args.steps)
  plan.close()

  # The batched value-and-gradient alone (the tensor-core part of a step).
  idx = torch.randint(0, MLP_N, (MLP_CHAINS, MLP_MB), dtype=torch.int32, device="cuda")
  for _ in range(3):
    pot.evaluate(Xd, idx, ds, grad=True)
  torch.cuda.synchronize()
  g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  reps = 10
  g0.record()
  for _ in range(reps):
    pot.evaluate(Xd, idx, ds, grad=True)
  g1.record()
  torch.cuda.synchronize()
  grad_ms = g0.elapsed_time(g1) / reps
  flops = MLP_CHAINS * MLP_FLOP_PER_GRAD
  achieved = flops / (grad_ms / 1e3) / 1e12
  peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
      if (ROOT / "MEASURED_PEAKS.json").exists() else {}
  peak = peaks.get("bf16_tflops_sustained", 1700.0)

  # Plain one-chain FP32 GPU form: the same network in torch fp32 ops,
  # differentiated by autograd, one OBABO step (two gradients) per chain.
  w = Xd[0].clone()
  p = torch.zeros_like(w)
  Xt = torch.from_numpy(X).cuda()
  yt = torch.from_numpy(y).cuda()

  def plain_grad(w, rows):
    w = w.detach().requires_grad_(True)
    q = lik.unravel(w)
    z1 = torch.tanh(Xt[rows] @ q["W1"] + q["b1"])
    z2 = torch.tanh(z1 @ q["W2"] + q["b2"])
    out = (z2 @ q["W3"])[:, 0] + q["b3"]
    lk = torch.distributions.Normal(out, 0.1).log_prob(yt[rows])
    U = -(MLP_N / MLP_MB) * lk.sum() + 0.5 * (w * w).sum()
    U.backward()
    return w.grad

  def plain_step():
    nonlocal w, p
    hh, keep = 1e-7, math.exp(-1e-7)
    p = math.sqrt(keep) * p + math.sqrt(1 - keep) * torch.randn_like(p)
    p = p - 0.5 * hh * plain_grad(w, torch.randint(0, MLP_N, (MLP_MB,), device="cuda"))
    w = w + hh * p
    p = p - 0.5 * hh * plain_grad(w, torch.randint(0, MLP_N, (MLP_MB,), device="cuda"))
    p = math.sqrt(keep) * p + math.sqrt(1 - keep) * torch.randn_like(p)

  for _ in range(3):
    plain_step()
  torch.cuda.synchronize()
  q0 = time.perf_counter()
  plain_n = 20
  for _ in range(plain_n):
    plain_step()
  torch.cuda.synchronize()
  plain_value = plain_n / (time.perf_counter() - q0)

  # End to end through alias.obabo: host samples in, one kept sample out.
  kw = dict(cache_size=64, batch_size=MLP_MB, integration_steps=10,
            friction=1.0, first_step_size=1e-7, last_step_size=1e-8)
  init_trees = [lik.unravel(inits[c]) for c in range(MLP_CHAINS)]
  alias.obabo(pot, loader, accepted_samples=1, **kw)(*init_trees[:2], iterations=2)
  its = max(2, args.steps // 10)
  torch.cuda.synchronize()
  s0 = time.perf_counter()
  res = alias.obabo(pot, loader, accepted_samples=1, **kw)(*init_trees, iterations=its)
  torch.cuda.synchronize()
  e2e_s = time.perf_counter() - s0
  e2e_value = MLP_CHAINS * its * 10 / e2e_s
  P = lik.param_count
  h2d = MLP_CHAINS * P * 4 / (its * 10)
  d2h = MLP_CHAINS * res[0]["sample_count"] * (P * 4 + 8) / (its * 10)

  cpu = None
  if rank == 0:
    threads = os.cpu_count() or 1
    g_rate = mlp_cpu_grad_rate(lik, X, y, inits, 3, threads)
    cpu = {"value": g_rate / 2.0, "unit": "chain-steps/s", "cores": threads,
           "kind": "port",
           "sample": f"3 float64 gradients of one chain (numpy oracle, {threads} "
                     "threads); an OBABO step is two gradients"}
  if rank == 0:
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "chain-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 GEMMs, f32 state",
        "data": "synthetic (teacher MLP targets, numpy default_rng(20261206)); "
                "X 144 MB resident in HBM",
        "config": {"workload": MLP_WORKLOAD, "n_obs": MLP_N, "chains_per_gpu": MLP_CHAINS,
                   "minibatch": MLP_MB, "integrator": "OBABO (2 gradients per step)",
                   "index_stream": "numpy PCG64 per chain, bit-exact",
                   "noise": "Philox4x32-10", "l2": "activations 1.4 GB per gradient, "
                   "larger than L2", "graph_block_steps": 50},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": "measured bf16_tflops_sustained",
                     "kernel": "batched value-and-gradient (5 tcgen05 GEMMs + "
                               "elementwise kernels), 64 chains",
                     "kernel_ms": grad_ms,
                     "algorithmic_flop_per_launch": flops},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "chain-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": "gbsgmc.alias.obabo(...)(*64 samples, iterations=K/10)"},
        "plain_gpu": {"value": plain_value, "unit": "chain-steps/s",
                      "form": "one chain, torch fp32 ops + autograd per gradient",
                      "fused_over_plain": value / world / plain_value},
        "clocks": clk, "finite": finite,
    }), flush=True)


def run_gemm(args):
  """The tcgen05 BF16 GEMM alone on the tanh network's hidden-layer shape,
  64 x (2048 x 1024 x 1024): C fp32 from the CTA-pair kernel and the
  single-CTA kernel (GBSGMC_GEMM_PAIR=0) in the four operand layouts, C BF16
  from both (K-major operands), and torch.bmm (cuBLAS, BF16 output) beside
  them; CUDA events over `--steps` calls after `--warmup`, one JSON line."""
  import os
  import torch
  from gbsgmc import _lib
  batch, M, N, K = 64, 2048, 1024, 1024
  flop = 2.0 * batch * M * N * K
  g = torch.Generator(device="cuda").manual_seed(5)
  A = torch.randn((batch, M, K), generator=g, device="cuda").to(torch.bfloat16)
  B = torch.randn((batch, N, K), generator=g, device="cuda").to(torch.bfloat16)
  At, Bt = A.transpose(1, 2).contiguous(), B.transpose(1, 2).contiguous()
  C = torch.empty((batch, M, N), device="cuda")
  status = torch.zeros(1, dtype=torch.int32, device="cuda")

  def timed(fn):
    for _ in range(args.warmup):
      fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
      fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / args.steps

  out = {}
  for pair in ("1", "0"):
    os.environ["GBSGMC_GEMM_PAIR"] = pair
    for a_mn, b_mn in ((0, 0), (0, 1), (1, 0), (1, 1)):
      Ap, Bp = (At if a_mn else A), (Bt if b_mn else B)

      def call():
        _lib.call("gbsgmc_gemm_bf16", a_mn, b_mn, Ap.data_ptr(), M if a_mn else K, M * K,
                  Bp.data_ptr(), N if b_mn else K, N * K, C.data_ptr(), N, M * N, batch,
                  M, N, K, status.data_ptr(), _lib.stream_handle())

      ms = timed(call)
      out[f"{'pair' if pair == '1' else 'single'}_{'mn' if a_mn else 'k'}{'mn' if b_mn else 'k'}"] = \
          round(flop / (ms / 1e3) / 1e12, 1)
  # BF16 C (as torch.bmm writes it): half the output bytes.
  C16 = torch.empty((batch, M, N), dtype=torch.bfloat16, device="cuda")
  for pair in ("1", "0"):
    os.environ["GBSGMC_GEMM_PAIR"] = pair

    def call16():
      _lib.call("gbsgmc_gemm_bf16_c16", 0, 0, A.data_ptr(), K, M * K, B.data_ptr(), K, N * K,
                C16.data_ptr(), N, M * N, batch, M, N, K, status.data_ptr(),
                _lib.stream_handle())

    ms = timed(call16)
    out[f"{'pair' if pair == '1' else 'single'}_kk_bf16_out"] = \
        round(flop / (ms / 1e3) / 1e12, 1)
  os.environ.pop("GBSGMC_GEMM_PAIR", None)
  assert int(status.item()) == 0
  ms = timed(lambda: torch.bmm(A, B.transpose(1, 2)))
  out["torch_bmm_bf16_out"] = round(flop / (ms / 1e3) / 1e12, 1)
  print(json.dumps({"metric": "bf16 GEMM throughput", "unit": "TFLOP/s",
                    "shape": {"batch": batch, "M": M, "N": N, "K": K},
                    "steps": args.steps, "warmup": args.warmup, "results": out}), flush=True)


def run_gather(args):
  """The headline kernel's memory pattern without its arithmetic: random
  1 KB rows (fp32, d = 256) of the 1,000,000-row matrix, 256 x 1024 per
  step, gathered by torch.index_select (a library kernel, for comparison
  only) and by a plain row copy with the same index stream; CUDA events
  over `--steps` steps after `--warmup`, one JSON line with GB/s and its
  fraction of the measured copy bandwidth."""
  import torch
  N, d, rows = 1_000_000, 256, 256 * 1024
  X = torch.randn((N, d), device="cuda")
  g = torch.Generator(device="cuda").manual_seed(3)
  idx = torch.randint(0, N, (args.warmup + args.steps, rows), generator=g, device="cuda")
  out = torch.empty((rows, d), device="cuda")

  def timed(fn):
    for k in range(args.warmup):
      fn(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.steps):
      fn(args.warmup + k)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / args.steps

  ms = timed(lambda k: torch.index_select(X, 0, idx[k], out=out))
  gbs = rows * d * 4 / (ms / 1e3) / 1e9
  peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
      if (ROOT / "MEASURED_PEAKS.json").exists() else {}
  peak = peaks.get("hbm_gbs", 6800.0)
  print(json.dumps({"metric": "random 1 KB row gather", "unit": "GB/s",
                    "rows_per_step": rows, "row_bytes": d * 4, "matrix_rows": N,
                    "steps": args.steps, "warmup": args.warmup,
                    "torch_index_select": {"GB/s": gbs, "frac_of_copy_peak": gbs / peak,
                                           "read_plus_write_GB/s": 2 * gbs,
                                           "ms_per_step": ms}}), flush=True)


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=K_CONFIG)
  ap.add_argument("--warmup", type=int, default=5)
  ap.add_argument("--impl", default="gbsgmc", choices=["gbsgmc", "reference"])
  ap.add_argument("--workload", default="logistic",
                  choices=["logistic", "mlp", "resgld", "cnn", "gemm", "gather"],
                  help="logistic: 256-chain SGLD headline; mlp: 64-chain OBABO "
                       "on the tanh network; resgld: 32-replica exchange on it; "
                       "cnn: 8-chain OBABO on the conv classifier; gemm: the "
                       "tcgen05 GEMM alone on the network's hidden-layer shape; "
                       "gather: the headline's random-row memory pattern alone")
  ap.add_argument("--kernel-only", action="store_true",
                  help="short run of the fused kernel for profilers; no JSON line")
  args = ap.parse_args()
  if args.warmup < 3:
    ap.error("--warmup must be at least 3")
  if args.workload == "gemm":
    run_gemm(args)
  elif args.workload == "gather":
    run_gather(args)
  elif args.workload == "cnn":
    if args.impl == "reference":
      run_mlp_reference(args)
    elif args.kernel_only:
      cnn_kernel_only(args)
    else:
      run_cnn(args)
  elif args.workload == "resgld":
    if args.impl == "reference":
      run_mlp_reference(args)
    else:
      run_resgld(args)
  elif args.workload == "mlp":
    if args.impl == "reference":
      run_mlp_reference(args)
    elif args.kernel_only:
      mlp_kernel_only(args)
    else:
      run_mlp(args)
  elif args.impl == "reference":
    run_reference(args)
  elif args.kernel_only:
    kernel_only(args)
  else:
    run_gbsgmc(args)


if __name__ == "__main__":
  main()
