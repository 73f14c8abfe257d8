"""Benchmark: NeuralODE forward+adjoint gradient evaluations per second on GB300.

Workload (the batched headline configuration): u0 in R^{64 x 16384} ~ N(0,1);
MLP 64->256->256->64 tanh with Glorot-uniform weights; tspan (0,1); 20 uniform
saveat points; Tsit5 abstol 1e-7 reltol 1e-5; targets from a seeded stable
linear ODE du/dt = M u (M = Q diag(-U(0.1,2)) Q^T); MSE loss;
InterpolatingAdjoint with checkpoints at the save points.

One step = one gradient evaluation: forward solve, fused MSE loss at the save
points, adjoint solve, parameter-gradient reduction.

  value : grad evals/s with inputs resident in HBM (device C-ABI entry points),
          device time from CUDA events on the library's stream.
  e2e   : the same through the host-pointer path a caller uses: every step copies
          u0 and the targets host->device from pinned memory and reads the loss
          and dL/dp back.

Multi-GPU: the reference couples the whole batch through one step-size
controller, so N > 1 runs N independent replicas (weak scaling, no collective
on the data path); `value` is the sum over ranks.

`--impl reference` times the CPU path on the host cores instead: the FP32 C++
restatement of the same algorithm (oracle/cpu_fp32.cpp; the reference's Julia
stack is not available on this machine), on the full batch, every step one
whole gradient evaluation, all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "diffeqflux.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "NeuralODE grad evals/sec, BF16-TC vs plain FP32 GPU, at <=1e-3 rel err vs FP64"
UNIT = "grad_evals/s"


def workload_name(B, S=64, H=256):
    return f"neuralode_b{B}_s{S}_h{H}x2_tanh_nsave20"


def glorot_params(dims, rng):
    """Flat parameters of Dense layers dims[0] -> ... -> dims[-1]: Glorot-uniform
    weights (column-major out x in, the ComponentArray order) and zero biases."""
    parts = []
    for i in range(len(dims) - 1):
        lim = np.sqrt(6.0 / (dims[i] + dims[i + 1]))
        W = rng.uniform(-lim, lim, size=(dims[i + 1], dims[i]))
        parts += [W.T.reshape(-1), np.zeros(dims[i + 1])]
    return np.concatenate(parts).astype(np.float32)


def workload(S=64, H=256, B=16384, nsave=20, seed=1):
    from scipy.linalg import expm
    rng = np.random.default_rng(seed)
    dims = [S, H, H, S]
    p = glorot_params(dims, rng)
    u0 = rng.standard_normal((S, B)).astype(np.float32)
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    M = Q @ np.diag(-rng.uniform(0.1, 2.0, S)) @ Q.T
    ts = np.linspace(0.0, 1.0, nsave)
    tgt = np.stack([expm(M * t) @ u0.astype(np.float64) for t in ts], axis=-1).astype(np.float32)
    return dict(S=S, H=H, B=B, dims=dims, p=p, u0=u0, ts=ts, target=tgt, tspan=(0.0, 1.0),
                abstol=1e-7, reltol=1e-5)


def gemm_flops_per_rhs(dims, B):
    return 2.0 * B * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms; start()
    returns once the first sample has arrived (at most 5 s), so the samples
    cover the timed region that follows it."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


class CpuArm:
    """The CPU path on the host cores: the FP32 C++ restatement of the same
    gradient evaluation (Tsit5 + PI controller + saveat, MSE, InterpolatingAdjoint;
    OpenMP over the batch, one thread per core), on the FULL batch -- no
    sampling, no scaling. It agrees with the FP64 oracle to ~1e-7 on the loss
    and both gradients, and takes the same accepted steps as the GPU forms."""

    def __init__(self, wl, B=None):
        from oracle import cpu_fp32
        self.wl = wl
        self.B = B or wl["B"]
        self.cores = host_cores()
        self.m = cpu_fp32.CpuNeuralODE(wl["dims"], [1] * (len(wl["dims"]) - 2) + [0], wl["p"], self.B,
                                       nthreads=self.cores)
        self.u0 = wl["u0"][:, :self.B]
        self.tg = wl["target"][:, :self.B, :]

    def grad_eval(self):
        wl = self.wl
        t0 = time.perf_counter()
        out = self.m.grad(self.u0, wl["tspan"], wl["ts"], wl["abstol"], wl["reltol"], self.tg, loss_kind=1)
        return time.perf_counter() - t0, out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = workload(S=args.state, H=args.hidden, B=args.batch)
    arm = CpuArm(wl)
    for _ in range(args.warmup):
        arm.grad_eval()
    t_all = time.perf_counter()
    secs = []
    out = None
    for _ in range(args.steps):
        sec, out = arm.grad_eval()
        secs.append(sec)
    wall = time.perf_counter() - t_all
    v = args.steps / sum(secs)
    loss, _, _, _, cnt = out
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(secs) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": workload_name(wl["B"], wl["S"], wl["H"]), "batch": wl["B"],
                   "state": wl["S"], "hidden": wl["H"], "nsave": 20, "abstol": 1e-7, "reltol": 1e-5,
                   "sensealg": "InterpolatingAdjoint", "loss": "MSE"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": arm.cores, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"full workload: every step one gradient evaluation of all {wl['B']} "
                                   f"trajectories (FP32 C++ restatement, OpenMP, {arm.cores} threads); "
                                   f"the reference's Julia stack is not installed on this machine"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "solver": {"nf_fwd": cnt["nf"], "naccept": cnt["naccept"], "nreject": cnt["nreject"],
                   "nf_adj": cnt["nf_adj"], "naccept_adj": cnt["naccept_adj"], "nreject_adj": cnt["nreject_adj"],
                   "loss": loss},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    return 0


class Form:
    """One precision form of the solver with its device buffers; ``grad_eval``
    is one training-step gradient: forward solve, fused MSE at the save
    points, adjoint solve (four kernel launches)."""

    LAUNCHES_PER_EVAL = 4   # forward, loss, adjoint, quadrature reduction

    def __init__(self, wl, precision, local, dev, u0_d, tg_d, p_d):
        import ctypes as C

        import torch

        import gbnde
        from gbnde import _lib
        S, B, H = wl["S"], wl["B"], wl["H"]
        model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
        self.solver = gbnde.Solver(model, precision, local)
        self.lib = self.solver.lib
        self.desc = gbnde.Solver.solve_desc(0.0, 1.0, wl["ts"], wl["abstol"], wl["reltol"], 0)
        ns = len(wl["ts"])
        self.u0_d, self.tg_d = u0_d, tg_d
        self.us_d = torch.empty((ns, B, S), dtype=torch.float32, device=dev)
        self.dl_d = torch.empty_like(self.us_d)
        self.du0_d = torch.empty((B, S), dtype=torch.float32, device=dev)
        self.dp_d = torch.empty(self.solver.nparams, dtype=torch.float32, device=dev)
        self.solver.set_params_device(p_d)
        torch.cuda.synchronize()
        # The library launches on a torch-owned stream: pinned-memory copies
        # issued on it stay valid however the objects are torn down (torch's
        # host allocator records events on every stream a pinned block was
        # used on, also when the block is freed).
        self.lstream = torch.cuda.Stream(device=dev)
        _lib.check(self.lib.gbnde_set_stream(self.solver.h, C.c_void_p(self.lstream.cuda_stream)))
        self.st_f, self.st_b, self.loss = _lib.Stats(), _lib.Stats(), C.c_double()
        self._C, self._check, self.S, self.B = C, _lib.check, S, B

    def grad_eval(self):
        C, lib, h = self._C, self.lib, self.solver.h
        self._check(lib.gbnde_forward_device(h, C.byref(self.desc), self.S, self.B,
                                             self.u0_d.data_ptr(), self.us_d.data_ptr(),
                                             C.byref(self.st_f)))
        self._check(lib.gbnde_loss_device(h, self.us_d.data_ptr(), self.tg_d.data_ptr(), 1,
                                          self.dl_d.data_ptr(), C.byref(self.loss)))
        self._check(lib.gbnde_backward_device(h, self.dl_d.data_ptr(), self.du0_d.data_ptr(),
                                              self.dp_d.data_ptr(), C.byref(self.st_b)))

    def timed(self, steps, flush):
        """Device time (ms) of `steps` gradient evaluations, L2 flushed before each."""
        import torch
        tot = 0.0
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.lstream)
            self.grad_eval()
            e1.record(self.lstream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return tot


# ---------------------------------------------------------------------------
# The other workloads, each through the host API a user calls (host arrays in
# and out, copies included), a few evaluations each: latency of the batch-1
# spiral fit, FFJORD at d = 16 / B = 65536, and uneven multiple shooting.
# The BF16 form covers widths <= 256 and no time input, so these run the FP32
# form.
# ---------------------------------------------------------------------------
def _timed(fn, n):
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(n):
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return sorted(ts)[len(ts) // 2]


def _kernel_ms(solver):
    import ctypes as C
    fm, bm = C.c_double(), C.c_double()
    solver.lib.gbnde_last_kernel_ms(solver.h, C.byref(fm), C.byref(bm))
    return fm.value, bm.value


def aux_spiral(device):
    """cube -> Dense(2, 50, tanh) -> Dense(50, 2), u0 = [2, 0], tspan (0, 1.5),
    30 save points, Tsit5 1e-7 / 1e-5, SSE loss, InterpolatingAdjoint; batch 1."""
    import gbnde
    rng = np.random.default_rng(0)
    model = gbnde.Chain(gbnde.cube(), gbnde.Dense(2, 50, "tanh"), gbnde.Dense(50, 2))
    p = model.init_params(rng)
    ts = np.linspace(0.0, 1.5, 30)
    node = gbnde.NeuralODE(model, (0.0, 1.5), gbnde.Tsit5("fp32"), saveat=ts, abstol=1e-7,
                           reltol=1e-5, sensealg=gbnde.InterpolatingAdjoint())
    s = node.solver
    s.set_params(p)
    from scipy.integrate import solve_ivp
    u0 = np.array([[2.0], [0.0]], np.float32)
    A = np.array([[-0.1, 2.0], [-2.0, -0.1]])
    # target: du/dt = A^T u.^3 (docs/src/examples/neural_ode.md:24-30) at 1e-10
    sol = solve_ivp(lambda t, u: A.T @ u ** 3, (0.0, 1.5), [2.0, 0.0], method="DOP853", t_eval=ts,
                    rtol=1e-10, atol=1e-10)
    tgt = sol.y[:, None, :].astype(np.float32)
    out = {}

    def step():
        us, st = s.forward(u0, node.desc())
        du0, dp, sb = s.backward((2.0 * (us - tgt)).astype(np.float32))
        out["st"], out["sb"] = st, sb
    sec = _timed(step, 20)
    kf, kb = _kernel_ms(s)
    # the CPU path on the same problem: the FP32 C++ restatement, one thread
    # (one trajectory leaves nothing to spread over cores)
    cpu = None
    try:
        from oracle import cpu_fp32
        m = cpu_fp32.CpuNeuralODE([2, 50, 2], [1, 0], p, 1, cube=True, nthreads=1)
        m.grad(u0, (0.0, 1.5), ts, 1e-7, 1e-5, tgt, loss_kind=0)
        reps = 20
        t0 = time.perf_counter()
        for _ in range(reps):
            m.grad(u0, (0.0, 1.5), ts, 1e-7, 1e-5, tgt, loss_kind=0)
        cpu = {"latency_ms": 1000.0 * (time.perf_counter() - t0) / reps, "cores": 1, "kind": "port",
               "cpu": cpu_model(), "sample": f"{reps} gradient evaluations (FP32 C++ restatement, one thread)"}
        m.close()
    except Exception as e:  # reported, never silently dropped
        cpu = {"error": f"{type(e).__name__}: {e}"}
    return {"workload": "spiral_b1_s2_cube_h50_nsave30", "latency_ms": 1000.0 * sec,
            "fwd_kernel_ms": kf, "bwd_kernel_ms": kb,
            "unit": "ms per gradient evaluation (forward + adjoint, host API)", "precision": "fp32",
            "nf_fwd": out["st"].nf, "nf_adj": out["sb"].nf_adj, "cpu": cpu,
            "note": "batch 1: latency-bound (launch and controller round trips), no roofline"}


def aux_ffjord(device, B=65536, d=16, H=512):
    """FFJORD, (d+1) -> H -> H -> d softplus with time input, B samples of a
    seeded 8-component Gaussian mixture, Hutchinson trace, Tsit5 1e-5 / 1e-5;
    negative log-likelihood and its adjoint gradient. The BF16 form (primal
    and tangent chains on the tensor cores) is the reported value; the FP32
    form runs the same inputs beside it and bounds its error."""
    import gbnde
    rng = np.random.default_rng(3)
    means = 2.0 * rng.standard_normal((8, d))
    var = rng.uniform(0.2, 1.0, (8, d))
    comp = rng.integers(0, 8, B)
    x = (means[comp] + np.sqrt(var[comp]) * rng.standard_normal((B, d))).T.astype(np.float32)
    model = gbnde.Chain(gbnde.Dense(d + 1, H, "softplus"), gbnde.Dense(H, H, "softplus"), gbnde.Dense(H, d))
    p = model.init_params(rng)
    noise = None
    g = (-np.ones(B) / B).astype(np.float32)
    F = gemm_flops_per_rhs([d + 1, H, H, d], B)
    res = {}
    for prec in ("bf16", "fp32"):
        fj = gbnde.FFJORD(model, (0.0, 1.0), (d,), gbnde.Tsit5(prec), abstol=1e-5, reltol=1e-5,
                          time_input=True)
        if noise is None:
            noise = fj.draw_noise(rng, B)
        out = {}

        def step():
            logpx, zT, st = fj.forward_np(x, p, noise)
            dx, dp, sb = fj.backward_np(g)
            out["st"], out["sb"], out["nll"], out["dp"] = st, sb, -float(np.mean(logpx)), dp
        sec = _timed(step, 2)
        kf, kb = _kernel_ms(fj.solver)
        st, sb = out["st"], out["sb"]
        # algorithmic GEMM work: a forward evaluation is the primal chain and
        # one Jacobian-vector chain (2F); an adjoint evaluation recomputes both
        # (2F), runs both chains backwards (2F) and forms the weight gradient (2F)
        flops = 2 * F * st.nf + 6 * F * sb.nf_adj
        res[prec] = {"value": 1.0 / sec, "ms_per_eval": 1000.0 * sec, "nf_fwd": st.nf, "nf_adj": sb.nf_adj,
                     "nll": out["nll"], "gemm_tflops_per_s": flops / sec / 1e12,
                     "fwd_kernel_ms": kf, "bwd_kernel_ms": kb,
                     "kernels": {"fwd": _lib_path_name(st.fwd_path), "adj": _lib_path_name(sb.adj_path)},
                     "dp": out["dp"]}
        fj.solver.close()
    tc, f32 = res["bf16"], res["fp32"]
    d_tc, d_32 = tc.pop("dp").astype(np.float64), f32.pop("dp").astype(np.float64)
    return {"workload": f"ffjord_b{B}_d{d}_h{H}x2_softplus", "value": tc["value"], "unit": "grad_evals/s",
            "precision": "bf16", **{k: v for k, v in tc.items() if k != "value"},
            "fp32_form": {**f32, "speedup_of_bf16_form": tc["value"] / f32["value"],
                          "nll_rel_diff": abs(tc["nll"] - f32["nll"]) / abs(f32["nll"]),
                          "grad_rel_diff": float(np.linalg.norm(d_tc - d_32) / np.linalg.norm(d_32))},
            "note": "host API (x, noise, logpx, gradients through host memory)"}


def aux_multishoot(device, ntraj=256, S=32, H=128):
    """Multiple shooting: ntraj trajectories of the oscillator network
    du/dt = -0.1 u + W tanh(u), W ~ N(0, 1/S), n_i ~ U{40..400} points at
    dt = 0.05, group sizes U{5..40}, continuity weight 100, MSE; every group of
    every trajectory in one launch; the loss gradient through the library's
    discrete adjoint."""
    import torch
    from scipy.integrate import solve_ivp

    import gbnde
    rng = np.random.default_rng(4)
    W = rng.standard_normal((S, S)) / np.sqrt(S)
    n = rng.integers(40, 401, ntraj)
    gs = rng.integers(5, 41, ntraj)
    T = 0.05 * (int(n.max()) - 1)
    y0 = rng.standard_normal((S, ntraj))

    def f(t, y):
        u = y.reshape(S, ntraj)
        return (-0.1 * u + W @ np.tanh(u)).ravel()
    tall = 0.05 * np.arange(int(n.max()))
    sol = solve_ivp(f, (0.0, T), y0.ravel(), method="DOP853", t_eval=tall, rtol=1e-8, atol=1e-10)
    Y = sol.y.reshape(S, ntraj, -1)
    trajs = [(Y[:, k, :n[k]].astype(np.float32), tall[:n[k]], int(gs[k])) for k in range(ntraj)]
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
    p0 = torch.from_numpy(model.init_params(rng)).to(torch.device("cuda", device))
    solver = gbnde.Solver(model, "fp32", device)
    out = {}

    def step():
        # mean of squares per group + default continuity loss: the fused device path
        p = p0.clone().requires_grad_(True)
        loss, _ = gbnde.multiple_shoot_batch(p, trajs, solver, gbnde.mse_loss, abstol=1e-6, reltol=1e-3)
        loss.backward()
        out["loss"] = float(loss.detach())
    sec = _timed(step, 5)
    kf, kb = _kernel_ms(solver)
    nseg = sum(len(gbnde.group_ranges(int(n[k]), int(gs[k]))) for k in range(ntraj))
    return {"workload": f"multishoot_{ntraj}traj_s{S}_h{H}x2_uneven", "value": 1.0 / sec,
            "unit": "grad_evals/s", "ms_per_eval": 1000.0 * sec, "precision": "fp32",
            "segments": nseg, "points": int(n.sum()), "loss": out["loss"],
            "fwd_kernel_ms": kf, "bwd_kernel_ms": kb,
            "note": "host API (data and parameters in, gradient out): the packed segments in one "
                    "forward launch, the loss and continuity terms in one loss kernel, one adjoint "
                    "launch from the device cotangent"}


# ---------------------------------------------------------------------------
# Sweep over (state, hidden width, batch): the training iteration (forward,
# fused MSE, adjoint, Adam) replayed as one CUDA graph per step, FP32 form
# with autotuned tiles and BF16 form where the engine covers the shape, and
# the FP64 oracle on a small sample of the same point. Bounded: a few steps
# per point (the configuration's 200 Adam steps are the same iteration).
# ---------------------------------------------------------------------------
SWEEP_S = (16, 64, 256)
SWEEP_H = (128, 512, 1024)
SWEEP_B = (1024, 16384, 262144)


def sweep_data(S, H, B, dev, seed=5, nsave=20):
    """u0 ~ N(0, 1), Glorot weights, targets of du/dt = M u with
    M = Q diag(-U(0.1, 2)) Q^T (exp(M t) from scipy, the products on the GPU)."""
    import torch
    from scipy.linalg import expm
    rng = np.random.default_rng(seed)
    dims = [S, H, H, S]
    p = glorot_params(dims, rng)
    Q, _ = np.linalg.qr(rng.standard_normal((S, S)))
    M = Q @ np.diag(-rng.uniform(0.1, 2.0, S)) @ Q.T
    ts = np.linspace(0.0, 1.0, nsave)
    g = torch.Generator(device=dev).manual_seed(seed)
    u0 = torch.randn((B, S), generator=g, device=dev, dtype=torch.float32)  # column-major S x B
    E = torch.from_numpy(np.stack([expm(M * t) for t in ts]).astype(np.float32)).to(dev)
    tg = torch.matmul(u0.unsqueeze(0), E.transpose(1, 2)).contiguous()      # nsave x B x S
    return dims, p, ts, u0, tg, E


def sweep_point(S, H, B, prec, dev, warmup, steps, tune):
    import torch

    import gbnde
    dims, p, ts, u0, tg, E = sweep_data(S, H, B, dev)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, H, "tanh"), gbnde.Dense(H, S))
    solver = gbnde.Solver(model, prec, dev.index or 0)
    desc = gbnde.Solver.solve_desc(0.0, 1.0, ts, 1e-7, 1e-5, 0)
    out = {"precision": prec}
    pd = torch.from_numpy(p).to(dev)
    solver.set_params_device(pd)
    if tune:
        out["tile_rows"] = list(solver.autotune(u0, desc, S, B))
    m, v = torch.zeros_like(pd), torch.zeros_like(pd)
    graphed = []
    for k in range(warmup):
        solver.graph_train_step(u0, tg, desc, S, B, pd, m, v, 1 + k, lr=1e-3, kind=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        loss, st, gd = solver.graph_train_step(u0, tg, desc, S, B, pd, m, v, 1 + warmup + k, lr=1e-3, kind=1)
        graphed.append(gd)
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t0) / steps
    F = gemm_flops_per_rhs(dims, B)
    flops = F * (st.nf + st.nf_recompute + 3 * (st.nf_adj - st.nf_adj_vjp) + 2 * st.nf_adj_vjp)
    out.update({"value": 1.0 / sec, "unit": "train_steps/s", "ms_per_step": 1000.0 * sec,
                "steps": steps, "replayed_as_graph": all(graphed), "loss": loss,
                "kernels": {"fwd": _lib_path_name(st.fwd_path), "adj": _lib_path_name(st.adj_path)},
                "nf_fwd": st.nf, "nf_adj": st.nf_adj, "gemm_tflops_per_s": flops / sec / 1e12})
    if prec == "bf16":
        # a step of seconds-long loops: against the sustained measured peak
        peak = measured_peaks().get("bf16_tflops_sustained")
        if peak:
            out["frac_of_bf16_peak_sustained"] = flops / sec / 1e12 / peak
    solver.close()
    return out, (dims, p, ts, u0, tg)


def _lib_path_name(code):
    from gbnde import _lib
    return _lib.PATH_NAMES.get(int(code), str(code))


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def run_sweep(args):
    """One JSON line per (state, hidden, batch) point."""
    import torch
    dev = torch.device("cuda", 0)
    pts = [(S, H, B) for B in SWEEP_B for S in SWEEP_S for H in SWEEP_H]
    if args.sweep_max_batch:
        pts = [x for x in pts if x[2] <= args.sweep_max_batch]
    if args.sweep_state:
        pts = [x for x in pts if x[0] == args.sweep_state]
    if args.sweep_hidden:
        pts = [x for x in pts if x[1] == args.sweep_hidden]
    for S, H, B in pts:
        line = {"sweep_point": {"state": S, "hidden": H, "batch": B}, "data": "synthetic (seeded)",
                "config": "NeuralODE S -> H -> H -> S tanh, tspan (0, 1), 20 saves, Tsit5 1e-7 / 1e-5, "
                          "MSE to a random stable linear ODE, InterpolatingAdjoint, Adam lr 1e-3"}
        big = B > 16384
        # the first graph step runs eagerly and captures, later ones replay;
        # at B = 262144 a step takes seconds, so one replayed step is timed
        warm, steps = (1, 1) if big else (2, 5)
        data = None
        for prec in ("fp32", "bf16"):
            if prec == "bf16" and not (S <= 256 and H <= 1024):
                line["bf16"] = {"unsupported": "the tensor-core engine covers state <= 256 and widths <= 1024"}
                continue
            try:
                r, data = sweep_point(S, H, B, prec, dev, warm, steps, tune=(prec == "fp32" and not big))
                line[prec] = r
            except Exception as e:  # reported per point
                line[prec] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
        if "value" in line.get("fp32", {}) and "value" in line.get("bf16", {}):
            line["bf16_over_fp32"] = line["bf16"]["value"] / line["fp32"]["value"]
        if data is not None and not args.no_cpu:
            dims, p, ts, u0, tg = data
            n = min(1024, B)
            wl = {"dims": dims, "p": p, "ts": ts, "abstol": 1e-7, "reltol": 1e-5, "B": B, "tspan": (0.0, 1.0),
                  "u0": u0[:n].T.cpu().numpy(), "target": tg[:, :n, :].permute(2, 1, 0).cpu().numpy()}
            arm = CpuArm(wl, B=n)
            sec, _ = arm.grad_eval()
            line["cpu"] = {"value": (n / B) / sec, "unit": "grad_evals/s", "cores": arm.cores, "kind": "port",
                           "sample": f"one gradient evaluation of {n} of {B} trajectories in {sec:.2f} s "
                                     f"(FP32 C++ restatement), scaled linearly to the batch"
                                     + ("" if n == B else " (the step count at the full batch may differ)")}
        del data
        torch.cuda.empty_cache()
        print(json.dumps(line), flush=True)
    return 0


def profiled_traffic(kernel, workload_name):
    """DRAM bytes per launch of `kernel` on `workload_name` from the committed
    ncu summaries: a line `traffic_bytes_per_launch <kernel> <workload> = N`."""
    import glob
    import re
    pat = re.compile(r"traffic_bytes_per_launch\s+(\S+)\s+(\S+)\s*=\s*([0-9.eE+]+)")
    for fn in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for ln in open(fn):
            m = pat.search(ln)
            if m and m.group(1) == kernel and m.group(2) == workload_name:
                return float(m.group(3)), os.path.relpath(fn, ROOT)
    return None, None


def run_gpu(args):
    import ctypes as C

    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    wl = workload(S=args.state, H=args.hidden, B=args.batch)
    S, B = wl["S"], wl["B"]
    dev = torch.device("cuda", local)
    ns = len(wl["ts"])
    # column-major device buffers
    u0_d = torch.from_numpy(np.ascontiguousarray(wl["u0"].T)).to(dev)
    tg_d = torch.from_numpy(np.ascontiguousarray(np.transpose(wl["target"], (2, 1, 0)))).to(dev)
    p_d = torch.from_numpy(wl["p"]).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    form = Form(wl, args.precision, local, dev, u0_d, tg_d, p_d)
    solver, lib, lstream = form.solver, form.lib, form.lstream
    st_f, st_b, loss = form.st_f, form.st_b, form.loss
    du0_d, dp_d = form.du0_d, form.dp_d
    grad_eval = form.grad_eval

    for _ in range(args.warmup):
        grad_eval()
    torch.cuda.synchronize()
    # ---- timed region: device-resident inputs ----------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    k_fwd = k_bwd = 0.0
    flops = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)           # L2 flush between steps (256 MB > 129 MB L2)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lstream)
        grad_eval()
        e1.record(lstream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        fm, bm = C.c_double(), C.c_double()
        lib.gbnde_last_kernel_ms(solver.h, C.byref(fm), C.byref(bm))
        k_fwd += fm.value
        k_bwd += bm.value
        F = gemm_flops_per_rhs(wl["dims"], B)
        # a full adjoint evaluation is 3F (recompute + two transpose products),
        # one that reuses the previous activations 2F
        flops_b = F * st_b.nf_recompute + 3.0 * F * (st_b.nf_adj - st_b.nf_adj_vjp) + 2.0 * F * st_b.nf_adj_vjp
        flops += flops_b
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    t_max = total_ms
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    ms_per_step = t_max / args.steps
    value = world * args.steps / (t_max / 1000.0)

    # ---- e2e: host buffers, copies inside the timed region ---------------------
    u0_h = torch.from_numpy(np.ascontiguousarray(wl["u0"].T)).pin_memory()
    tg_h = torch.from_numpy(np.ascontiguousarray(np.transpose(wl["target"], (2, 1, 0)))).pin_memory()
    dp_h = torch.empty(solver.nparams, dtype=torch.float32).pin_memory()
    h2d = u0_h.numel() * 4 + tg_h.numel() * 4
    d2h = dp_h.numel() * 4 + 8
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e_ms = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lstream)
        with torch.cuda.stream(lstream):
            u0_d.copy_(u0_h, non_blocking=True)
            tg_d.copy_(tg_h, non_blocking=True)
        grad_eval()
        with torch.cuda.stream(lstream):
            dp_h.copy_(dp_d, non_blocking=True)
        e1.record(lstream)
        e1.synchronize()
        e_ms += e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e_ms = float(t.item())
    e2e = world * args.steps / (e_ms / 1000.0)

    peaks = measured_peaks()
    peak_tf = peaks.get("bf16_tflops", 1900.0)
    peak_src = "measured" if "bf16_tflops" in peaks else "fallback"
    bwd_ms_avg = k_bwd / args.steps
    wide = args.precision == "bf16" and (S > 64 or wl["H"] > 256)
    kname = ("bwd_tcw_kernel" if wide else "bwd_tc_kernel") if args.precision == "bf16" else "bwd_f32_kernel"
    traffic, traffic_src = profiled_traffic(kname, workload_name(B, S, wl["H"]))
    achieved_tf = (flops / args.steps) / (bwd_ms_avg / 1000.0) / 1e12
    roof = {"kernel": kname,
            "bound": "tensor", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": achieved_tf / peak_tf, "peak_source": peak_src,
            "traffic": traffic, "traffic_source": traffic_src,
            "basis": "GEMM FLOPs of the adjoint launch: F*nf_recompute + 3F*(nf_adj - nf_adj_vjp) + "
                     "2F*nf_adj_vjp (VJP-only evaluations reuse the activations), F = 2*B*sum(in*out)"}

    # ---- the training iteration as one CUDA graph (gbnde_graph_train_step) -------
    # forward, loss, adjoint and Adam (lr 1e-3) replayed as one graph from the
    # second call on; auxiliary figure (the working set, about 1 GB of stage
    # storage and images, exceeds L2, so no flush between steps)
    graph = None
    if not args.no_graph:
        pg = p_d.clone()
        mg = torch.zeros_like(pg)
        vg = torch.zeros_like(pg)
        flags = []
        for st_i in (1, 2):
            solver.graph_train_step(u0_d, tg_d, form.desc, S, B, pg, mg, vg, st_i, lr=1e-3, kind=1)
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(lstream)
        for k in range(args.steps):
            lg, sg, gd = solver.graph_train_step(u0_d, tg_d, form.desc, S, B, pg, mg, vg, 3 + k, lr=1e-3, kind=1)
            flags.append(gd)
        g1.record(lstream)
        g1.synchronize()
        gms = g0.elapsed_time(g1) / args.steps
        graph = {"value": 1000.0 / gms, "unit": "train_steps/s", "ms_per_step": gms, "steps": args.steps,
                 "all_replayed_as_graph": all(flags), "last_loss": lg,
                 "note": "forward + fused MSE + adjoint + Adam per step, one CUDA graph launch each"}
        solver.set_params_device(p_d)
        torch.cuda.synchronize()

    # ---- the plain FP32 form on the same inputs: speed ratio and agreement ------
    fp32 = None
    if args.precision == "bf16" and not args.no_fp32_form:
        g_tc = dp_d.double().cpu().numpy()
        loss_tc = loss.value
        f32 = Form(wl, "fp32", local, dev, u0_d, tg_d, p_d)
        tiles32 = f32.solver.autotune(f32.u0_d, f32.desc, wl["S"], wl["B"])
        f32.grad_eval()
        torch.cuda.synchronize()
        n32 = max(1, min(args.steps, 3))
        ms32 = f32.timed(n32, flush) / n32
        g32 = f32.dp_d.double().cpu().numpy()
        fp32 = {"value": 1000.0 / ms32, "ms_per_step": ms32, "steps": n32,
                "speedup_of_bf16_form": (value / world) * ms32 / 1000.0,
                "loss_rel_diff": abs(loss_tc - f32.loss.value) / abs(f32.loss.value),
                "grad_rel_diff": float(np.linalg.norm(g_tc - g32) / np.linalg.norm(g32)),
                "autotuned_tile_rows": {"forward": tiles32[0], "adjoint": tiles32[1]},
                "note": "plain FP32 kernels, same inputs; the FP32 form agrees with the FP64 "
                        "oracle to ~1e-6, so the differences bound the BF16 form's error"}
        del f32

    aux = None
    if rank == 0 and not args.no_aux:
        aux = {}
        for name, fn in (("spiral", aux_spiral), ("ffjord", aux_ffjord), ("multiple_shooting", aux_multishoot)):
            if args.aux and name != args.aux:
                continue
            try:
                aux[name] = fn(local)
            except Exception as e:  # reported, never silently dropped
                aux[name] = {"error": f"{type(e).__name__}: {e}"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        arm = CpuArm(wl)
        secs = []
        while not secs or (sum(secs) < args.cpu_seconds and len(secs) < 3):
            secs.append(arm.grad_eval()[0])
        v = len(secs) / sum(secs)
        cpu = {"value": v, "unit": UNIT, "cores": arm.cores, "kind": "port", "cpu": cpu_model(),
               "sample": f"{len(secs)} full gradient evaluation(s) of all {B} trajectories in "
                         f"{sum(secs):.1f} s (FP32 C++ restatement, OpenMP, {arm.cores} threads)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
        "data": "synthetic (seeded)",
        "config": {"workload": workload_name(B, S, wl["H"]), "batch": B, "state": S,
                   "hidden": wl["H"], "nsave": ns, "abstol": 1e-7, "reltol": 1e-5,
                   "sensealg": "InterpolatingAdjoint", "loss": "MSE", "precision": args.precision,
                   "l2": "flushed between steps (256 MB write)", "parallelism": "replicas"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps * Form.LAUNCHES_PER_EVAL,
        "fp32_form": fp32,
        "graph_train_step": graph,
        "other_workloads": aux,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "solver": {"nf_fwd": st_f.nf, "naccept": st_f.naccept, "nreject": st_f.nreject,
                   "nf_recompute": st_b.nf_recompute, "nf_adj": st_b.nf_adj, "nf_adj_vjp": st_b.nf_adj_vjp,
                   "naccept_adj": st_b.naccept_adj, "nreject_adj": st_b.nreject_adj,
                   "fwd_kernel_ms": k_fwd / args.steps, "bwd_kernel_ms": bwd_ms_avg,
                   "loss": loss.value},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["fp32", "bf16"])
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--state", type=int, default=64, help="state dim of the NeuralODE (headline: 64)")
    ap.add_argument("--hidden", type=int, default=256, help="width of its two hidden layers (headline: 256)")
    ap.add_argument("--aux", default="", choices=["", "spiral", "ffjord", "multiple_shooting"],
                    help="run only this one of the other workloads")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="the GPU line's cpu_baseline: full gradient evaluations until this many seconds (1-3)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32-form", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-aux", action="store_true", help="skip the spiral, FFJORD and multiple-shooting figures")
    ap.add_argument("--sweep", action="store_true", help="state x hidden x batch sweep, one JSON line per point")
    ap.add_argument("--sweep-max-batch", type=int, default=0)
    ap.add_argument("--sweep-state", type=int, default=0, help="only this state dim")
    ap.add_argument("--sweep-hidden", type=int, default=0, help="only this hidden width")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.sweep:
        return run_sweep(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
