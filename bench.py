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
  from oracle import sgmc_oracle as O
  st = O.loader_rng(seed).bit_generator.state
  s, inc = st["state"]["state"], st["state"]["inc"]
  m = (1 << 64) - 1
  return [(s >> 64) & m, s & m, (inc >> 64) & m, inc & m, 0]


def dist_env():
  rank = int(os.environ.get("RANK", "0"))
  world = int(os.environ.get("WORLD_SIZE", "1"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  return rank, world, local


class Clocks:
  """Samples nvidia-smi clocks and throttle reasons during the timed region."""
  QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, gpu_index):
    self.gpu = gpu_index
    self.proc = None

  def start(self):
    try:
      self.proc = subprocess.Popen(
          ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
           "--format=csv,noheader,nounits", "-lms", "100"],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except (OSError, ValueError):
      self.proc = None

  def stop(self):
    if self.proc is None:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    self.proc.terminate()
    try:
      out, _ = self.proc.communicate(timeout=5)
    except subprocess.TimeoutExpired:
      self.proc.kill()
      out, _ = self.proc.communicate()
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
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


def measured_peak_hbm():
  p = ROOT / "MEASURED_PEAKS.json"
  if p.exists():
    try:
      return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except (KeyError, ValueError):
      pass
  return 6800.0, "fallback"


def profiled_traffic():
  """DRAM bytes per launch of the fused step from the committed ncu summary."""
  p = ROOT / "profiles" / "glm_sgld_step_logistic_256x1024x256.md"
  if not p.exists():
    return None
  for line in p.read_text().splitlines():
    if line.startswith("traffic_bytes_per_launch:"):
      try:
        return float(line.split(":", 1)[1].strip().split()[0])
      except ValueError:
        return None
  return None


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
    self.chain_base = rank * CHAINS
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
  """Direct launches of the fused step kernel on torch's current stream."""

  def __init__(self, s):
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

  def __call__(self, i):
    L = self._lib
    L.call("gbsgmc_sgld_glm_step", self.model, CHAINS, MB, L.ptr(self.idx[i % 8]),
           MB, L.ptr(self.W), L.ptr(self.V), 0.9, 1e-5, self.sched, self.noise,
           None, None, None, None, L.ptr(self.ws), self.ws.numel(),
           L.ptr(self.status), self.stream)


def kernel_only(args):
  """A short run for profilers: three plan steps, ten more, then five direct
  launches of the fused step kernel."""
  import torch
  rank, _, local = dist_env()
  torch.cuda.set_device(local)
  s = Setup(rank)
  plan = s.plan(args.warmup + 10)
  plan.run(0, args.warmup)
  plan.run(args.warmup, 10)
  torch.cuda.synchronize()
  plan.check_status()
  plan.close()
  f = FusedLauncher(s)
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
  plan = s.plan(args.warmup + args.steps)

  # W untimed warm-up steps, then exactly K timed steps (device events).
  plan.run(0, args.warmup)
  barrier()
  clocks = Clocks(local)
  clocks.start()
  start = torch.cuda.Event(enable_timing=True)
  end = torch.cuda.Event(enable_timing=True)
  barrier()
  start.record()
  plan.run(args.warmup, args.steps)
  end.record()
  barrier()
  clk = clocks.stop()
  ms = start.elapsed_time(end)
  plan.check_status()
  if world > 1:
    t = torch.tensor([ms], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
  value = world * CHAINS * args.steps / (ms / 1e3)
  launches = plan.launches(args.steps)
  shape = plan.launch_shape()
  finite = bool(torch.isfinite(s.W).all().item())
  plan.close()

  # The fused step kernel alone: average launch time on its stream.
  f = FusedLauncher(s)
  for i in range(5):
    f(i)
  reps = 200
  torch.cuda.synchronize()
  k0 = torch.cuda.Event(enable_timing=True)
  k1 = torch.cuda.Event(enable_timing=True)
  k0.record()
  for i in range(reps):
    f(i)
  k1.record()
  torch.cuda.synchronize()
  kernel_ms = k0.elapsed_time(k1) / reps
  bytes_per_launch = CHAINS * BYTES_PER_CHAIN_STEP
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
  alias.sgld(s.pot, s.loader, accepted_samples=1, **kw)(
      *init[:2], iterations=args.warmup)          # warm the path
  e2e_run = alias.sgld(s.pot, s.loader, accepted_samples=min(1000, args.steps),
                       **kw)
  barrier()
  e0 = time.perf_counter()
  results = e2e_run(*init, iterations=args.steps)
  barrier()
  e2e_s = time.perf_counter() - e0
  kept = results[0]["sample_count"]
  h2d = CHAINS * (D * 4 + 40) + args.steps * 12
  d2h = CHAINS * kept * (D * 4 + 8)
  e2e_value = world * CHAINS * args.steps / e2e_s

  # CPU oracle on a bounded sample (rank 0 only).
  cpu = None
  if rank == 0:
    threads = os.cpu_count() or 1
    val, _ = cpu_chain_steps(s.X, s.y, 2 * threads, 2, threads)
    cpu = {"value": val, "unit": "chain-steps/s", "cores": threads,
           "kind": "port",
           "sample": f"{2 * threads} chains x 2 steps (numpy restatement, "
                     f"{threads} threads)"}

  if rank == 0:
    line = {
        "metric": METRIC, "value": value, "unit": "chain-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (numpy default_rng(20261205); X 1.02 GB resident in HBM)",
        "config": {"workload": WORKLOAD, "n_obs": N_OBS, "d": D,
                   "chains_per_gpu": CHAINS, "minibatch": MB,
                   "index_stream": "numpy PCG64 per chain, bit-exact",
                   "noise": "Philox4x32-10",
                   "l2": "inputs larger than L2 (X 1.02 GB, random rows)",
                   "parallelism": f"chains sharded, {world} replica(s)",
                   "graph_block_steps": 50,
                   "launch_shape": {"ctas_per_chain": shape[0],
                                    "rows_per_warp": shape[1],
                                    "warps_per_cta": shape[2],
                                    "chosen_by": "autotuner"}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic(),
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
        "clocks": clk, "finite": finite,
        "device_status": int(f.status.item()),
    }
    print(json.dumps(line), flush=True)
  if world > 1:
    dist.destroy_process_group()


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=K_CONFIG)
  ap.add_argument("--warmup", type=int, default=5)
  ap.add_argument("--impl", default="gbsgmc", choices=["gbsgmc", "reference"])
  ap.add_argument("--kernel-only", action="store_true",
                  help="short run of the fused kernel for profilers; no JSON line")
  args = ap.parse_args()
  if args.warmup < 3:
    ap.error("--warmup must be at least 3")
  if args.impl == "reference":
    run_reference(args)
  elif args.kernel_only:
    kernel_only(args)
  else:
    run_gbsgmc(args)


if __name__ == "__main__":
  main()
