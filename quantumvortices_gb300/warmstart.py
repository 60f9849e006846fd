"""Learned ARGLE warm-start (new; the reference has no machine learning).

A conv encoder-decoder (libvk's tcgen05 BF16 kernels, vk_nn_*) maps the
seeded vortex phase ansatz plus a signed vortex-charge density to a
correction of the ansatz; ARGLE (vk_argle) then continues from the
corrected field.  Training data are generated by the solver itself:
each sample is (ansatz, ARGLE-relaxed state).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import vk


class WarmStartNet:
    """The network; batch > 1 sizes it for batches of that many images
    (forward / loss_grad / train_step then take the images set by
    set_batch, [b][3][h][w] inputs and [b][2][h][w] targets).  The network
    runs on its own CUDA stream and every call returns with that stream
    synchronised; tensors produced by torch kernels must be complete (e.g.
    torch.cuda.current_stream().synchronize()) before they are passed in."""

    def __init__(self, h: int, w: int, base: int = 32, levels: int = 4, seed: int = 1, batch: int = 1):
        self.lib = vk.load_library()
        L = self.lib
        dp, vp = C.POINTER(C.c_double), C.c_void_p
        fp = C.POINTER(C.c_float)
        for name, res, args in [
            ("vk_nn_create", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(vp)]),
            ("vk_nn_create_batched", C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                               C.POINTER(vp)]),
            ("vk_nn_set_batch", C.c_int, [vp, C.c_int32]),
            ("vk_nn_features", C.c_int, [vp, dp, dp, C.c_int32, C.c_double, C.c_void_p]),
            ("vk_nn_destroy", C.c_int, [vp]),
            ("vk_nn_num_params", C.c_int, [vp, C.POINTER(C.c_int64)]),
            ("vk_nn_get_params", C.c_int, [vp, fp, C.c_int64]),
            ("vk_nn_set_params", C.c_int, [vp, fp, C.c_int64]),
            ("vk_nn_forward", C.c_int, [vp, C.c_void_p, C.c_void_p, vp]),
            ("vk_nn_loss_grad", C.c_int, [vp, C.c_void_p, C.c_void_p, dp, fp]),
            ("vk_nn_train_step", C.c_int, [vp, C.c_void_p, C.c_void_p, C.c_float, dp]),
        ]:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        self.h, self.w, self.base, self.levels = h, w, base, levels
        self.capacity, self.batch = batch, batch
        hnd = C.c_void_p()
        vk._check(L.vk_nn_create_batched(h, w, base, levels, batch, seed, C.byref(hnd)), "vk_nn_create_batched")
        self._h = hnd
        n = C.c_int64()
        vk._check(L.vk_nn_num_params(self._h, C.byref(n)), "vk_nn_num_params")
        self.nparam = int(n.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            vk._check(self.lib.vk_nn_destroy(self._h), "vk_nn_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_batch(self, b: int) -> None:
        vk._check(self.lib.vk_nn_set_batch(self._h, int(b)), "vk_nn_set_batch")
        self.batch = int(b)

    def features(self, psi: np.ndarray, pos: np.ndarray, width: float, out_dev) -> None:
        """Input features of one image on the GPU (vk_nn_features): out_dev, a
        CUDA float32 tensor [3,h,w], gets Re/Im psi and the signed Gaussian
        vortex-charge density of the positions pos[n, 2] (+ for the first half)."""
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        q = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 2)
        vk._check(self.lib.vk_nn_features(self._h, vk._dptr(a.view(np.float64)), vk._dptr(q), len(q), float(width),
                                          out_dev.data_ptr()), "vk_nn_features")

    def get_params(self) -> np.ndarray:
        a = np.empty(self.nparam, dtype=np.float32)
        vk._check(self.lib.vk_nn_get_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float)), self.nparam), "get")
        return a

    def set_params(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float32)
        vk._check(self.lib.vk_nn_set_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float)), self.nparam), "set")

    def forward(self, inp_dev, out_dev) -> None:
        """inp_dev/out_dev: torch CUDA float32 tensors [3,h,w] / [2,h,w]."""
        vk._check(self.lib.vk_nn_forward(self._h, inp_dev.data_ptr(), out_dev.data_ptr(), None), "vk_nn_forward")

    def loss_grad(self, inp_dev, tgt_dev):
        loss = C.c_double()
        g = np.empty(self.nparam, dtype=np.float32)
        vk._check(self.lib.vk_nn_loss_grad(self._h, inp_dev.data_ptr(), tgt_dev.data_ptr(), C.byref(loss),
                                           g.ctypes.data_as(C.POINTER(C.c_float))), "vk_nn_loss_grad")
        return float(loss.value), g

    def train_step(self, inp_dev, tgt_dev, lr: float, want_loss: bool = False):
        loss = C.c_double()
        vk._check(self.lib.vk_nn_train_step(self._h, inp_dev.data_ptr(), tgt_dev.data_ptr(), lr,
                                            C.byref(loss) if want_loss else None), "vk_nn_train_step")
        return float(loss.value) if want_loss else None


def _torch():
    import torch  # device memory and plumbing only; the network runs in libvk
    return torch


class DataGen:
    """Solver-generated training pairs: (features, relaxed - ansatz)."""

    def __init__(self, n: int, relax_steps: int = 1000, dt: float = 1e-3, precision: int = vk.VK_PREC_FP32):
        self.n, self.relax, self.dt = n, relax_steps, dt
        self.params = vk.params_for(n, dt=dt, precision=precision, otoc=True)
        self.solver = vk.GPESolver(self.params)
        dx = 2 * math.pi / n
        self.xi0 = math.sqrt(2.0) * dx
        self.width = 2.0 * self.xi0

    def ansatz(self, nv: int, seed: int):
        pos = self.solver.set_psi_vortices(nv, seed, self.xi0, min_sep=4 * self.xi0)
        return pos, self.solver.get_psi()

    def sample(self, nv: int, seed: int, net: "WarmStartNet"):
        """(features [3,n,n], relaxed - ansatz [2,n,n]) as CUDA float32 tensors;
        the features come from the network's feature kernel."""
        torch = _torch()
        pos, psi0 = self.ansatz(nv, seed)
        self.solver.argle(self.relax)
        # relaxed state = F^-1[kpsi] (psi itself is one step behind after
        # ARGLE): vk_set_kpsi transforms it on the device
        self.solver.set_kpsi(self.solver.get_kpsi())
        d = self.solver.get_psi() - psi0
        feat = torch.empty((3, self.n, self.n), dtype=torch.float32, device="cuda")
        net.features(psi0, pos, self.width, feat)
        tgt = torch.from_numpy(np.stack([d.real, d.imag]).astype(np.float32)).cuda()
        return feat, tgt

    def close(self):
        self.solver.close()


def vortex_count(rng) -> int:
    return int(rng.integers(4, 65)) * 2  # 8..128, even (neutral)


def generate(net: WarmStartNet, gen: DataGen, n_train: int, seed0: int = 10_000, log=print):
    """n_train solver-generated samples (seeds seed0..seed0+n_train-1), kept on
    the GPU as float16 [n_train, 3, n, n] features and [n_train, 2, n, n]
    targets (the network rounds its input to BF16 anyway)."""
    torch = _torch()
    rng = np.random.default_rng(seed0)
    n = gen.n
    feats = torch.empty((n_train, 3, n, n), dtype=torch.float16, device="cuda")
    tgts = torch.empty((n_train, 2, n, n), dtype=torch.float16, device="cuda")
    t0 = time.perf_counter()
    for i in range(n_train):
        f, t = gen.sample(vortex_count(rng), seed0 + i, net)
        feats[i] = f
        tgts[i] = t
        # the copies must finish before the network stream reuses f's memory
        torch.cuda.current_stream().synchronize()
    torch.cuda.synchronize()
    tgen = time.perf_counter() - t0
    log(f"generated {n_train} ARGLE-relaxed {n}^2 samples in {tgen:.1f} s")
    return feats, tgts, tgen


def train(net: WarmStartNet, gen: DataGen, n_train: int, epochs: int, lr: float, seed0: int = 10_000,
          log=print, data=None):
    """Generates n_train samples (or takes data = (feats, tgts, gen_s)) and
    trains with batches of net.capacity images: one Adam step per batch, the
    learning rate halved every epoch."""
    torch = _torch()
    feats, tgts, tgen = data if data is not None else generate(net, gen, n_train, seed0, log)
    n_train = feats.shape[0]
    B = net.capacity
    net.set_batch(B)
    rng = np.random.default_rng(seed0 + 1)
    t0 = time.perf_counter()
    hist = []
    nstep = 0
    for ep in range(epochs):
        order = torch.from_numpy(rng.permutation(n_train)).cuda()
        tot, cnt = 0.0, 0
        for k in range(0, n_train - B + 1, B):
            idx = order[k:k + B]
            xb = feats.index_select(0, idx).float()
            yb = tgts.index_select(0, idx).float()
            # the network runs on its own stream: the batch must be complete
            torch.cuda.current_stream().synchronize()
            l = net.train_step(xb, yb, lr * (0.5 ** ep), want_loss=(nstep % 16 == 0))
            nstep += 1
            if l is not None:
                tot += l
                cnt += 1
        hist.append(tot / max(1, cnt))
        log(f"epoch {ep}: mean sampled loss {hist[-1]:.4e}")
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    fl = train_flops(net) * B
    return {"gen_s": tgen, "train_s": ts, "loss": hist, "flops_per_step": fl, "batch": B, "steps": nstep,
            "tensor_tflops": fl * nstep / ts / 1e12}


def train_flops(net: WarmStartNet) -> float:
    """Multiply-add FLOPs of one training step's convolutions (forward, data
    and weight gradients; the first layer has no data gradient)."""
    b, L = net.base, net.levels
    convs = [(3, b, 0), (b, b, 0)]
    for lv in range(1, L):
        convs += [(b << (lv - 1), b << lv, lv), (b << lv, b << lv, lv)]
    for lv in range(L - 2, -1, -1):
        convs += [(b << (lv + 1), b << lv, lv), (b << lv, b << lv, lv)]
    convs.append((b, 2, 0))
    tot = 0.0
    for i, (ci, co, lv) in enumerate(convs):
        npix = (net.h >> lv) * (net.w >> lv)
        f = 2.0 * npix * 9 * ci * co
        tot += f * (2 if i == 0 else 3)
    return tot


def steps_to(solver: vk.GPESolver, target: float, max_steps: int, chunk: int = 10):
    """ARGLE in chunks until the last-step residual <= target; returns
    (steps, residual).  Residual = ||kpsi_new-kpsi_old||/(dt ||kpsi_old||)."""
    steps, r = 0, float("inf")
    while steps < max_steps:
        r = solver.argle(chunk)
        steps += chunk
        if r <= target:
            break
    return steps, r


def _timed_argle(gen: DataGen, psi, steps: int) -> float:
    torch = _torch()
    gen.solver.set_psi(psi)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gen.solver.argle(steps)
    return time.perf_counter() - t0


def _grand(d) -> float:
    """The functional ARGLE descends: E - Omega N = etot - echem in the
    reference's normalisation (etot = egrad + eintr alone is not monotone
    under ARGLE, because the norm is free)."""
    return d.etot - d.echem


def evaluate(net: WarmStartNet, gen: DataGen, seeds, log=print):
    """Plain ARGLE from the ansatz vs ARGLE from the network's warm start.

    Residual criterion: the residual plain ARGLE reaches after gen.relax
    steps (the configured relaxation length); both starts run ARGLE in
    chunks of 10 until they reach it.  Times are wall times of one vk_argle
    call of the needed length (warm start: plus the network and its copy).
    Energy criterion: the ARGLE functional E - Omega N after gen.relax steps
    from either start, and the steps the warm start needs to reach plain
    ARGLE's value (chunks of gen.relax // 20, capped at 4 * gen.relax)."""
    torch = _torch()
    rng = np.random.default_rng(12345)
    out = []
    s = gen.solver
    n = gen.n
    net.set_batch(1)
    corr = torch.empty((2, n, n), device="cuda", dtype=torch.float32)
    feat = torch.empty((3, n, n), device="cuda", dtype=torch.float32)
    for seed in seeds:
        nv = vortex_count(rng)
        pos, psi0 = gen.ansatz(nv, seed)
        r_target = s.argle(gen.relax)
        d = s.diagnostics_gpe()
        e_plain, f_plain = d.etot, _grand(d)
        gen.ansatz(nv, seed)
        k_plain, _ = steps_to(s, r_target, gen.relax)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net.features(psi0, pos, gen.width, feat)
        net.forward(feat, corr)
        c = corr.cpu().numpy()
        t_net = time.perf_counter() - t0
        warm = psi0 + (c[0] + 1j * c[1])
        s.set_psi(warm)
        k_warm, r_warm = steps_to(s, r_target, 4 * gen.relax)
        t_plain = _timed_argle(gen, psi0, k_plain)
        t_warm = _timed_argle(gen, warm, k_warm) + t_net
        s.set_psi(warm)
        s.argle(gen.relax)
        d = s.diagnostics_gpe()
        e_warm, f_warm = d.etot, _grand(d)
        s.set_psi(warm)
        k_f, chunk = 0, max(10, gen.relax // 20)
        while k_f < 4 * gen.relax:
            s.argle(chunk)
            k_f += chunk
            if _grand(s.diagnostics_gpe()) <= f_plain:
                break
        out.append({"seed": int(seed), "nv": nv, "r_target": r_target, "plain_steps": k_plain,
                    "warm_steps": k_warm, "warm_reached": bool(r_warm <= r_target), "plain_s": t_plain,
                    "warm_s": t_warm, "net_s": t_net, "energy_plain": e_plain, "energy_warm_same_steps": e_warm,
                    "grand_plain": f_plain, "grand_warm_same_steps": f_warm,
                    "warm_steps_to_plain_grand": k_f})
        log(out[-1])
    return out


def summarize(rows):
    ps = np.array([r["plain_steps"] for r in rows], float)
    ws = np.array([r["warm_steps"] for r in rows], float)
    pt = np.array([r["plain_s"] for r in rows])
    wt = np.array([r["warm_s"] for r in rows])
    de = np.array([abs(r["energy_warm_same_steps"] - r["energy_plain"]) / abs(r["energy_plain"]) for r in rows])
    dg = np.array([(r["grand_warm_same_steps"] - r["grand_plain"]) / abs(r["grand_plain"]) for r in rows])
    kf = np.array([r["warm_steps_to_plain_grand"] for r in rows], float)
    return {"seeds": len(rows), "plain_steps_mean": float(ps.mean()), "warm_steps_mean": float(ws.mean()),
            "iterations_saved_frac": float(1 - ws.sum() / ps.sum()), "plain_s_mean": float(pt.mean()),
            "warm_s_mean": float(wt.mean()), "time_ratio_warm_over_plain": float(wt.sum() / pt.sum()),
            "time_ratio_median": float(np.median(wt / pt)),
            "reached_frac": float(np.mean([r["warm_reached"] for r in rows])),
            "rel_energy_diff_same_steps_mean": float(de.mean()),
            "rel_grand_diff_same_steps_mean": float(dg.mean()),
            "grand_lower_frac": float(np.mean(dg <= 0)),
            "warm_steps_to_plain_grand_median": float(np.median(kf))}


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train and evaluate the learned ARGLE warm start")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--relax", type=int, default=1000)
    ap.add_argument("--train", type=int, default=512)
    ap.add_argument("--eval", type=int, default=32)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--base", type=int, default=32)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    gen = DataGen(a.n, a.relax)
    net = WarmStartNet(a.n, a.n, a.base, a.levels, seed=1, batch=a.batch)
    tr = train(net, gen, a.train, a.epochs, a.lr)
    held = list(range(900_000, 900_000 + a.eval))  # disjoint from the training seeds
    rows = evaluate(net, gen, held)
    res = {"config": vars(a), "train": tr, "summary": summarize(rows), "rows": rows}
    print(json.dumps(res["summary"]))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f, indent=1)
    net.close()
    gen.close()


if __name__ == "__main__":
    main()
