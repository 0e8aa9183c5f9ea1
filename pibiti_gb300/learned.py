"""The learned corrector: training data, training and evaluation.

A coarse step is one SPH step with the time step multiplied by SUBSTEPS (4);
its force pass also writes 16 features per particle (density, pressure,
neighbour count, velocity divergence, kernel-weighted relative velocity and
position moments, SPH velocity increment, soft-wall velocity increment).  The MLP (16 -> 64 -> 64 -> 3,
BF16 tensor-core kernels in csrc/sph_mlp.cu) predicts the difference between
SUBSTEPS plain steps of dt and the coarse step, as a velocity correction in
units of |g| dt_coarse.

Training data comes from the batched ensemble (configs.ensemble): from a state
of the fine-dt run, one featured coarse step and SUBSTEPS fine steps give one
(features, target) pair per particle.  Then, for a few rounds, the states the
learned integrator itself visits are labelled the same way and added (the
network then learns to correct the states its own errors lead to).  Training runs the project's own
forward/backward kernels (sph_mlp_train_pass_tc, on tcgen05) with Adam (sph_mlp_adam).
Device buffers are torch tensors passed by pointer.
"""
from __future__ import annotations

import ctypes
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

SUBSTEPS = 4
HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_PATH = os.path.join(HERE, "models", "corrector.npz")


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@dataclass
class Model:
    params: np.ndarray      # 5443 FP32
    feat_mean: np.ndarray   # 16
    feat_std: np.ndarray    # 16
    out_scale: np.ndarray   # 3
    info: dict

    def save(self, path: str = MODEL_PATH) -> None:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez(path, params=self.params, feat_mean=self.feat_mean, feat_std=self.feat_std,
                 out_scale=self.out_scale, info=np.array(repr(self.info)))

    @classmethod
    def load(cls, path: str = MODEL_PATH) -> "Model":
        with np.load(path, allow_pickle=False) as z:
            return cls(z["params"].astype(np.float32), z["feat_mean"].astype(np.float32),
                       z["feat_std"].astype(np.float32), z["out_scale"].astype(np.float32),
                       {"saved": str(z["info"])})

    def install(self, sph: SPH) -> None:
        stats = np.concatenate([self.feat_mean, 1.0 / self.feat_std]).astype(np.float32)
        prm = np.ascontiguousarray(self.params, np.float32)
        osc = np.ascontiguousarray(self.out_scale, np.float32)
        _lib.check(_lib.lib().sph_learned_set_model(
            sph._h, ctypes.c_void_p(prm.ctypes.data), ctypes.c_void_p(stats.ctypes.data),
            ctypes.c_void_p(osc.ctypes.data)))


def learned_step(sph: SPH, coarse_steps: int, substeps: int = SUBSTEPS, tol: float = 0.01) -> int:
    """Coarse steps with the MLP correction; returns the number of fallbacks."""
    fb = ctypes.c_uint32()
    _lib.check(_lib.lib().sph_learned_step(sph._h, coarse_steps, substeps, tol, ctypes.byref(fb)))
    return fb.value


def set_options(sph: SPH, drift: float = -1.0, jerk: float = 0.0) -> None:
    """Factors of the coarse step's drift (position) and jerk (velocity)
    corrections: negative for (n-1)/(2n), 0 for none."""
    _lib.check(_lib.lib().sph_learned_set_options(sph._h, drift, jerk))


def features_step(sph: SPH, feat, ids, substeps: int = SUBSTEPS) -> None:
    _lib.check(_lib.lib().sph_features_step(sph._h, substeps, _p(feat), _p(ids)))


def _g_dt(params_list, sizes, substeps, torch):
    vals = []
    for p, n in zip(params_list, sizes):
        g = float(np.sqrt(p.gravity.x ** 2 + p.gravity.y ** 2 + p.gravity.z ** 2)) + 1e-6
        vals.append(np.full(n, g * p.timeStep * substeps, np.float32))
    return torch.from_numpy(np.concatenate(vals)).cuda()


def generate(xmls, pos, vel, sizes, snapshots: int = 8, warm: int = 20, gap: int = 20,
             substeps: int = SUBSTEPS):
    """(features [M,16], targets [M,3]) on the GPU from `snapshots` states of
    the fine-dt run of the given scenes."""
    import torch
    ps = [Scene.parse(x).params for x in xmls]
    fine, coarse = SPH(ps), SPH(ps)
    fine.set_array(ARRAY_POS, pos)
    fine.set_array(ARRAY_VEL, vel)
    fine.update(warm)
    n = fine.n
    gdt = _g_dt(ps, sizes, substeps, torch)
    tp = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    tv = torch.empty_like(tp)
    vc = torch.empty_like(tp)
    vf = torch.empty_like(tp)
    feats, targets = [], []
    for _ in range(snapshots):
        fine.get_array(ARRAY_POS, tp)
        fine.get_array(ARRAY_VEL, tv)
        torch.cuda.synchronize()
        coarse.set_array(ARRAY_POS, tp)
        coarse.set_array(ARRAY_VEL, tv)
        f = torch.empty((n, 16), dtype=torch.float32, device="cuda")
        ids = torch.empty(n, dtype=torch.int32, device="cuda")
        features_step(coarse, f, ids, substeps)
        coarse.get_array(ARRAY_VEL, vc)
        fine.update(substeps)
        fine.get_array(ARRAY_VEL, vf)
        torch.cuda.synchronize()
        t = (vf - vc)[:, :3] / gdt[:, None]
        idx = ids.long()
        feats.append(f)
        targets.append(t[idx].contiguous())
        fine.update(gap)
    fine.close()
    coarse.close()
    return torch.cat(feats), torch.cat(targets)


# Snapshot phases of the shipped model's training data: (snapshots, warm-up
# steps, steps between snapshots) of the fine run; the first covers the
# early collapse of each dam break, the second the rest of 2000 steps.
PHASES = ((6, 20, 30), (9, 220, 200))


def generate_rollout(model: "Model", xmls, pos, vel, sizes, snapshots: int = 8, warm: int = 20,
                     gap: int = 60, substeps: int = SUBSTEPS, drift: float = -1.0):
    """Like generate(), but from the states the learned integrator itself
    visits: the scenes advance with learned_step (`gap` coarse steps between
    snapshots, no density check), and each snapshot is labelled with one
    featured coarse step and `substeps` fine steps from that state."""
    import torch
    ps = [Scene.parse(x).params for x in xmls]
    lrn, fine, coarse = SPH(ps), SPH(ps), SPH(ps)
    lrn.set_array(ARRAY_POS, pos)
    lrn.set_array(ARRAY_VEL, vel)
    lrn.update(warm)
    model.install(lrn)
    set_options(lrn, drift)
    n = lrn.n
    gdt = _g_dt(ps, sizes, substeps, torch)
    tp = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    tv = torch.empty_like(tp)
    vc = torch.empty_like(tp)
    vf = torch.empty_like(tp)
    feats, targets = [], []
    for _ in range(snapshots):
        learned_step(lrn, gap, substeps, 1e9)
        lrn.get_array(ARRAY_POS, tp)
        lrn.get_array(ARRAY_VEL, tv)
        torch.cuda.synchronize()
        for h in (coarse, fine):
            h.set_array(ARRAY_POS, tp)
            h.set_array(ARRAY_VEL, tv)
        f = torch.empty((n, 16), dtype=torch.float32, device="cuda")
        ids = torch.empty(n, dtype=torch.int32, device="cuda")
        features_step(coarse, f, ids, substeps)
        coarse.get_array(ARRAY_VEL, vc)
        fine.update(substeps)
        fine.get_array(ARRAY_VEL, vf)
        torch.cuda.synchronize()
        t = (vf - vc)[:, :3] / gdt[:, None]
        feats.append(f)
        targets.append(t[ids.long()].contiguous())
    for h in (lrn, fine, coarse):
        h.close()
    return torch.cat(feats), torch.cat(targets)


def generate_phases(xmls, pos, vel, sizes, phases=PHASES, substeps: int = SUBSTEPS):
    """generate() over several snapshot phases, concatenated."""
    import torch
    fs, ts = [], []
    for snaps, warm, gap in phases:
        f, t = generate(xmls, pos, vel, sizes, snapshots=snaps, warm=warm, gap=gap,
                        substeps=substeps)
        fs.append(f)
        ts.append(t)
    return torch.cat(fs), torch.cat(ts)


def train(feats, targets, epochs: int = 6, batch: int = 65536, lr: float = 2e-3, seed: int = 0,
          log=None) -> Model:
    """Adam on the project's MLP kernels; returns the trained model."""
    import torch
    L = _lib.lib()
    mean = feats.mean(0)
    std = feats.std(0) + 1e-6
    x = ((feats - mean) / std).to(torch.bfloat16).view(torch.int16).contiguous()
    out_scale = targets.std(0) + 1e-9
    # the rare very large targets (stiff wall contacts) are clipped at 4 sigma
    t = (targets / out_scale).clamp(-4.0, 4.0).contiguous()
    rng = np.random.default_rng(seed)
    parts = []
    for k_in, k_out in ((16, 64), (64, 64), (64, 3)):
        parts.append(rng.normal(0, 1.0 / np.sqrt(k_in), size=(k_in, k_out)).ravel())
        parts.append(np.zeros(k_out))
    prm = torch.from_numpy(np.concatenate(parts).astype(np.float32)).cuda()
    m, v, grad = torch.zeros_like(prm), torch.zeros_like(prm), torch.zeros_like(prm)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    img = torch.zeros(L.sph_mlp_packed_bytes(), dtype=torch.uint8, device="cuda")
    _lib.check(L.sph_mlp_pack(_p(prm), _p(img), None))
    n = x.shape[0]
    step = 0
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=gen)
        lr_ep = lr * (0.5 ** max(0, ep - epochs // 2))
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            xb, tb = x[idx].contiguous(), t[idx].contiguous()
            grad.zero_()
            loss.zero_()
            _lib.check(L.sph_mlp_train_pass_tc(_p(img), _p(xb), _p(tb), batch, _p(grad), _p(loss), None))
            step += 1
            _lib.check(L.sph_mlp_adam(_p(prm), _p(m), _p(v), _p(grad), lr_ep, 0.9, 0.999, 1e-8,
                                      step, None))
            _lib.check(L.sph_mlp_pack(_p(prm), _p(img), None))
            tot += loss.item()
            cnt += 1
        history.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: mean loss {history[-1]:.4f}")
    return Model(prm.cpu().numpy(), mean.cpu().numpy(), std.cpu().numpy(),
                 out_scale.cpu().numpy(), {"loss_history": history, "samples": int(n)})


def zero_model() -> Model:
    """A network whose output is zero: the learned step then reduces to the
    coarse step with the drift correction and the density check."""
    return Model(np.zeros(_lib.lib().sph_mlp_param_count(), np.float32), np.zeros(16, np.float32),
                 np.ones(16, np.float32), np.ones(3, np.float32), {"zero": True})


def one_step_errors(model: Model, xml: str, pos, vel, warm: int = 40,
                    substeps: int = SUBSTEPS) -> dict:
    """Errors of one coarse step against `substeps` fine steps from the same
    state: mean |dv| (m/s) and mean |dx| (m) over particles, for the coarse
    step alone, with the drift correction, and with drift and network."""
    p = Scene.parse(xml).params
    pc = p.copy()
    pc.timeStep = p.timeStep * substeps
    with SPH(p) as fine:
        fine.set_array(ARRAY_POS, pos)
        fine.set_array(ARRAY_VEL, vel)
        fine.update(warm)
        s_pos, s_vel = fine.get_array(ARRAY_POS), fine.get_array(ARRAY_VEL)
        fine.update(substeps)
        xf, vf = fine.get_array(ARRAY_POS), fine.get_array(ARRAY_VEL)
    out = {}
    for name in ("coarse", "drift", "learned"):
        with SPH(pc if name == "coarse" else p) as h:
            h.set_array(ARRAY_POS, s_pos)
            h.set_array(ARRAY_VEL, s_vel)
            if name == "coarse":
                h.update(1)
            else:
                (model if name == "learned" else zero_model()).install(h)
                learned_step(h, 1, substeps, tol=1e9)
            x, v = h.get_array(ARRAY_POS), h.get_array(ARRAY_VEL)
        out[f"dv_{name}"] = float(np.abs(v[:, :3] - vf[:, :3]).sum(1).mean())
        out[f"dx_{name}"] = float(np.abs(x[:, :3] - xf[:, :3]).sum(1).mean())
    return out


def rollout(model: Model, xml: str, pos, vel, fine_steps: int, substeps: int = SUBSTEPS,
            tol: float = 0.01, warm: int = 0, drift: float = -1.0, jerk: float = 0.0,
            trace: int = 0) -> dict:
    """Mean-density trajectories of the fine-dt plain run, the coarse run,
    the coarse run with the drift correction (no network, no check) and the
    learned run, sampled every `substeps` fine steps.  Errors are relative to
    the fine run (max and mean over the samples); times are wall clock of
    the fine and the learned run, each including one stats read per sample.
    With trace = k, every k-th sample of each relative error is returned too."""
    import torch
    p = Scene.parse(xml).params
    pc = p.copy()
    pc.timeStep = p.timeStep * substeps
    coarse_steps = fine_steps // substeps
    out = {}
    with SPH(p) as fine:
        fine.set_array(ARRAY_POS, pos)
        fine.set_array(ARRAY_VEL, vel)
        if warm:
            fine.update(warm)
        s_pos, s_vel = fine.get_array(ARRAY_POS), fine.get_array(ARRAY_VEL)
        rho_f = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(coarse_steps):
            fine.update(substeps)
            rho_f.append(fine.stats()[0][1])
        out["fine_s"] = time.perf_counter() - t0
    rho = {}
    with SPH(pc) as c:
        c.set_array(ARRAY_POS, s_pos)
        c.set_array(ARRAY_VEL, s_vel)
        rho["coarse"] = []
        for _ in range(coarse_steps):
            c.update(1)
            rho["coarse"].append(c.stats()[0][1])
    with SPH(p) as d:
        d.set_array(ARRAY_POS, s_pos)
        d.set_array(ARRAY_VEL, s_vel)
        zero_model().install(d)
        set_options(d, drift, jerk)
        rho["drift"] = []
        for _ in range(coarse_steps):
            learned_step(d, 1, substeps, 1e9)
            rho["drift"].append(d.stats()[0][1])
    with SPH(p) as lrn:
        lrn.set_array(ARRAY_POS, s_pos)
        lrn.set_array(ARRAY_VEL, s_vel)
        model.install(lrn)
        set_options(lrn, drift, jerk)
        learned_step(lrn, 0, substeps, tol)  # allocations outside the timed loop
        rho["learned"], fb = [], 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(coarse_steps):
            fb += learned_step(lrn, 1, substeps, tol)
            rho["learned"].append(lrn.stats()[0][1])
        out["learned_s"] = time.perf_counter() - t0
    rho_f = np.asarray(rho_f)
    if trace:
        out["trace_rho_fine"] = [round(float(x), 3) for x in rho_f[trace - 1::trace]]
    for k, r in rho.items():
        e = np.abs(np.asarray(r) - rho_f) / rho_f
        out[f"err_{k}_max"] = float(e.max())
        out[f"err_{k}_mean"] = float(e.mean())
        if trace:
            out[f"trace_{k}"] = [round(float(x), 5) for x in e[trace - 1::trace]]
    out.update({"fallbacks": int(fb), "coarse_steps": coarse_steps,
                "speedup": out["fine_s"] / out["learned_s"],
                "rho_fine_end": float(rho_f[-1]), "rho_learned_end": float(rho["learned"][-1])})
    return out


def mlp_bench(model: Model, rows: int, reps: int = 20, seed: int = 0) -> dict:
    """The mma.sync and the tcgen05 forward pass (sph_mlp_forward,
    sph_mlp_forward_tc) on `rows` standard-normal BF16 feature rows with the
    model's weights: median CUDA-event time of `reps` launches each (L2
    flushed before each), and whether the outputs are bit-identical."""
    import torch
    L = _lib.lib()
    prm = torch.from_numpy(model.params).cuda()
    img = torch.zeros(L.sph_mlp_packed_bytes(), dtype=torch.uint8, device="cuda")
    _lib.check(L.sph_mlp_pack(_p(prm), _p(img), None))
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((rows, 16), generator=g, device="cuda").to(torch.bfloat16).view(torch.int16)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = {"rows": rows}
    ys = {}
    for name, fn in (("mma_sync", L.sph_mlp_forward), ("tcgen05", L.sph_mlp_forward_tc)):
        y = torch.zeros((rows, 3), dtype=torch.float32, device="cuda")
        _lib.check(fn(_p(img), _p(x), rows, _p(y), None))
        ts = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(fn(_p(img), _p(x), rows, _p(y), None))
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e3)
        out[f"{name}_us"] = sorted(ts)[len(ts) // 2]
        ys[name] = y
    status = ctypes.c_uint32(0)
    _lib.check(L.sph_mlp_status(ctypes.byref(status)))
    out["identical"] = bool(torch.equal(ys["mma_sync"], ys["tcgen05"]))
    out["tc_status"] = status.value
    return out


def main(argv=None) -> int:
    """python -m pibiti_gb300.learned train|evaluate [--scenes S] ..."""
    import argparse
    import json
    import sys
    import torch
    from . import configs
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "evaluate", "profile", "mlp-bench"],
                    help="profile: a few learned coarse steps on the 1M double dam break "
                         "(a short run for a profiler's launch list); mlp-bench: the two "
                         "forward kernels on --rows standard-normal feature rows")
    ap.add_argument("--steps", type=int, default=3, help="coarse steps of `profile`")
    ap.add_argument("--rows", type=int, default=1 << 20, help="rows of `mlp-bench`")
    ap.add_argument("--reps", type=int, default=20, help="timed launches of `mlp-bench`")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=16)
    ap.add_argument("--batch", type=int, default=32768)
    ap.add_argument("--rounds", type=int, default=2,
                    help="rounds of training on the learned integrator's own states")
    ap.add_argument("--fine-steps", type=int, default=2000)
    ap.add_argument("--model", default=MODEL_PATH)
    a = ap.parse_args(argv)
    log = lambda *m: print(*m, file=sys.stderr, flush=True)  # noqa: E731
    torch.cuda.set_device(0)
    if a.cmd == "train":
        e = configs.ensemble(scenes=a.scenes)
        t0 = time.perf_counter()
        f, t = generate_phases(e.xmls, e.pos, e.vel, e.sizes)
        log(f"generated {f.shape[0]} samples in {time.perf_counter() - t0:.1f} s")
        t0 = time.perf_counter()
        model = train(f, t, epochs=a.epochs, batch=a.batch, log=log)
        feats, targets = [f], [t]
        for rnd in range(a.rounds):
            # the states the current model's integrator visits, labelled by fine steps
            fr, tr = generate_rollout(model, e.xmls, e.pos, e.vel, e.sizes, snapshots=10, warm=20,
                                      gap=50)
            feats.append(fr)
            targets.append(tr)
            log(f"round {rnd + 1}: {sum(x.shape[0] for x in feats)} samples")
            model = train(torch.cat(feats), torch.cat(targets), epochs=a.epochs, batch=a.batch,
                          log=log)
        model.info.update({"scenes": a.scenes, "phases": PHASES, "epochs": a.epochs,
                           "batch": a.batch, "rounds": a.rounds,
                           "train_s": time.perf_counter() - t0})
        model.save(a.model)
        w = configs.dambreak_small(side=32, seed=9)
        print(json.dumps({"trained": model.info,
                          "one_step_32k": one_step_errors(model, w.xml, w.pos, w.vel)}))
    elif a.cmd == "profile":
        model = Model.load(a.model)
        w = configs.dambreak_double()
        with SPH(Scene.parse(w.xml).params) as s:
            s.set_array(ARRAY_POS, w.pos)
            s.set_array(ARRAY_VEL, w.vel)
            s.update(20)
            model.install(s)
            learned_step(s, 1, SUBSTEPS, 1e9)  # allocations
            s.update(2)
            fb = learned_step(s, a.steps, SUBSTEPS, 1e9)
            torch.cuda.synchronize()
        print(json.dumps({"profile": "done", "coarse_steps": a.steps, "fallbacks": fb}))
    elif a.cmd == "mlp-bench":
        print(json.dumps(mlp_bench(Model.load(a.model), a.rows, a.reps)))
    else:
        model = Model.load(a.model)
        w = configs.dambreak_double()
        print(json.dumps({"one_step_1M": one_step_errors(model, w.xml, w.pos, w.vel),
                          "rollout_1M": rollout(model, w.xml, w.pos, w.vel, a.fine_steps)}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
