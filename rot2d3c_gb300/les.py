"""Learned-closure experiment: DNS -> filtered training data -> CNN -> LES.

1. A fine FP32 run (DNS) on nf^2 with time-constant random-phase forcing in
   the shell 4-6 is spun up and sampled: every ``snap_every`` CFL steps the
   state is filtered onto the coarse nc^2 grid (sharp cutoff k <= nc/3) and
   the 8 network inputs and the 2 subgrid bracket tendencies are stored
   (``r2d3c_closure_sample``).
2. The closure CNN is trained on random batches with Adam (inputs and targets
   standardised per channel).
3. Starting from the filtered DNS state, three coarse runs advance over the
   same physical time as the continued DNS: the LES with the CNN tendencies
   (re-evaluated at every step), the plain coarse solver, and the fallback
   with hyperviscosity (nn > 1).  Their time-averaged energy spectra are
   compared with the filtered DNS spectrum for k <= k_c, and the GPU time per
   unit of physical time of the LES is compared with the DNS's.

No counterpart in the reference program.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import DT_CFL, FP32, Context, make_params
from .closure import CNN, closure_advance, closure_sample


def _field(n, kmin, kmax, amp_slope, rng):
    h = n // 2
    ka = np.concatenate([np.arange(h), np.arange(h) - h]).astype(np.float64)
    kx = ka[: h + 1]
    ka2 = kx[:, None] ** 2 + ka[None, :] ** 2
    k = np.sqrt(ka2)
    shell = (k >= kmin) & (k <= kmax)
    a = np.where(shell, np.where(k > 0, k, 1.0) ** amp_slope, 0.0) * np.exp(
        1j * rng.uniform(0, 2 * np.pi, size=ka2.shape))
    col = a[0]
    j = np.arange(1, h)
    col[n - j] = np.conj(col[j])
    col[0] = col[0].real
    col[h] = 0.0
    a[0] = col
    return a, ka2


def _energy(a, ka2, kin, n):
    two = np.full((a.shape[0], 1), 2.0)
    two[0, 0] = 1.0
    return float(np.sum(two * np.abs(a) ** 2 * ka2 ** kin) / float(n) ** 4)


def _setup_run(n, seed):
    """k^-2 / k^-1 initial ps, vz in shells 1-10 (energies 1/2 each) and a
    random-phase forcing in the shell 4-6 of unit energy."""
    rng = np.random.default_rng(seed)
    ps, ka2 = _field(n, 1.0, 10.0, -2.0, rng)
    vz, _ = _field(n, 1.0, 10.0, -1.0, rng)
    fp, _ = _field(n, 4.0, 6.0, 0.0, rng)
    fz, _ = _field(n, 4.0, 6.0, 0.0, rng)
    ps *= math.sqrt(0.5 / _energy(ps, ka2, 1, n))
    vz *= math.sqrt(0.5 / _energy(vz, ka2, 0, n))
    fp *= math.sqrt(1.0 / _energy(fp, ka2, 1, n))
    fz *= math.sqrt(1.0 / _energy(fz, ka2, 0, n))
    return ps, vz, fp, fz


def coarse_forcing(fp, fz, nf, nc):
    """The DNS forcing (shell 4-6) on the coarse grid."""
    h = nc // 2
    out = []
    for f in (fp, fz):
        g = np.zeros((h + 1, nc), np.complex128)
        for j in range(nc):
            ky = j if j < h else j - nc
            g[:h, j] = f[:h, ky if ky >= 0 else nf + ky] * (nc / nf) ** 2
        out.append(g)
    return out


def run_experiment(nf=2048, nc=256, omega=1.0, nu=2e-5, nsnap=1000, snap_every=10, spinup=2000,
                   train_steps=3000, batch=32, lr=1e-3, les_steps=4000, cfl=0.5, seed=1,
                   fallback_nn=4, spec_every=50, hnu=0.1):
    """Runs the three stages and returns a dict of timings and errors.

    nf, nc: DNS and LES grids; nu: viscosity of both (nn = 1); omega:
    rotation rate; hnu: large-scale (hypo)viscosity of all runs (mm = 2);
    nsnap snapshots taken every snap_every DNS steps after spinup steps; train_steps Adam steps of batch snapshots; les_steps coarse
    CFL steps, whose second half is averaged for the spectra (one spectrum
    every spec_every steps).  The fallback run replaces the viscosity by a
    hyperviscosity of order fallback_nn with the damping rate 20 nu k_c^2
    at the cutoff k_c = nc/3.
    """
    import torch

    les_steps = max(spec_every, les_steps // spec_every * spec_every)
    t_all = time.perf_counter()
    ps, vz, fp, fz = _setup_run(nf, seed)
    pf = make_params(n=nf, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0,
                     cfl=cfl)
    fine = Context(pf, FP32)
    fine.set_state(ps, vz)
    fine.set_forcing(fp, fz)
    fine.set_time(0.0)
    t_dns, _ = fine.advance(spinup, DT_CFL, cfl)
    # ---- 1. training data
    pc = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0,
                     cfl=cfl)
    coarse = Context(pc, FP32)
    X = torch.empty((nsnap, nc, nc, 8), dtype=torch.float32, device="cuda")
    Y = torch.empty((nsnap, nc, nc, 2), dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    for i in range(nsnap):
        t_dns, _ = fine.advance(snap_every, DT_CFL, cfl)
        closure_sample(fine, coarse, X[i], Y[i])
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    # ---- 2. training
    net = CNN(nc, nc, batch, seed)
    im, isd = X.mean(dim=(0, 1, 2)).cpu().numpy(), X.std(dim=(0, 1, 2)).cpu().numpy()
    om, osd = Y.mean(dim=(0, 1, 2)).cpu().numpy(), Y.std(dim=(0, 1, 2)).cpu().numpy()
    net.set_normalization(im, np.maximum(isd, 1e-12), om, np.maximum(osd, 1e-12))
    bx = torch.empty((batch, nc, nc, 8), dtype=torch.float32, device="cuda")
    by = torch.empty((batch, nc, nc, 2), dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    ntrain = max(1, int(0.9 * nsnap))
    losses = []
    t0 = time.perf_counter()
    for s in range(train_steps):
        idx = torch.randint(0, ntrain, (batch,), device="cuda", generator=gen)
        torch.index_select(X, 0, idx, out=bx)
        torch.index_select(Y, 0, idx, out=by)
        losses.append(net.train_step(bx, by, batch, lr))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # held-out loss (standardised units)
    val = []
    for i in range(ntrain, nsnap, batch):
        b = min(batch, nsnap - i)
        val.append(net.gradients(X[i:i + b].contiguous(), Y[i:i + b].contiguous(), b)[0])
    # ---- 3. LES vs plain vs hyperviscous fallback vs filtered DNS
    cfp, cfz = coarse_forcing(fp, fz, nf, nc)
    runs = {}
    for name, nn_, nuc in (("les", 1, nu), ("plain", 1, nu), ("fallback", fallback_nn, None)):
        p = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=nn_, mm=2, nnv=nn_, mmv=2, omega=omega, iflow=0,
                        cfl=cfl)
        if nuc is None:  # hyperviscosity with the same damping rate at the coarse cutoff
            kc = nc / 3.0
            p.nu = p.nuv = nu * kc ** 2 / kc ** (2 * nn_) * 20.0
        c = Context(p, FP32)
        runs[name] = c
    spectra = {k: [] for k in runs}
    spectra["dns"] = []
    fluxes = {k: [] for k in spectra}

    def flux(c):  # running sum of the total energy transfer (2-D part + vz part)
        _, f1, f2 = c.transfers()
        return np.cumsum(f1 + f2)
    xbuf = torch.empty((1, nc, nc, 8), dtype=torch.float32, device="cuda")
    tbuf = torch.empty((1, nc, nc, 2), dtype=torch.float32, device="cuda")
    # initial coarse state = filtered DNS state (through one closure sample)
    closure_sample(fine, coarse, xbuf[0], tbuf[0])
    ps_c, vz_c = coarse.get_state()
    t_dns0 = t_dns
    for name, c in runs.items():
        c.set_state(ps_c, vz_c)
        c.set_forcing(cfp, cfz)
        c.set_time(t_dns0)
    # LES with the CNN: closure evaluated at every step
    les = runs["les"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_les = t_dns0
    for s in range(0, les_steps, spec_every):
        t_les, _ = closure_advance(les, net, spec_every, DT_CFL, cfl)
        if s + spec_every > les_steps // 2:
            spectra["les"].append(les.spectrum()[0])
            fluxes["les"].append(flux(les))
    torch.cuda.synchronize()
    t_les_gpu = time.perf_counter() - t0
    T = t_les - t_dns0
    for name in ("plain", "fallback"):
        c = runs[name]
        for s in range(0, les_steps, spec_every):
            c.advance(spec_every, DT_CFL, cfl)
            if s + spec_every > les_steps // 2:
                spectra[name].append(c.spectrum()[0])
                fluxes[name].append(flux(c))
    # DNS over the same physical time; filtered spectrum sampled on the same
    # cadence in time
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    td = t_dns0
    dns_steps = 0
    nxt = t_dns0 + T / 2
    dT = T / 2 / max(1, len(spectra["les"]))
    while td < t_dns0 + T:
        td, _ = fine.advance(8, DT_CFL, cfl)
        dns_steps += 8
        if td >= nxt:
            closure_sample(fine, coarse, xbuf[0], tbuf[0])
            spectra["dns"].append(coarse.spectrum()[0])
            fluxes["dns"].append(flux(fine))
            nxt += dT
    torch.cuda.synchronize()
    t_dns_gpu = time.perf_counter() - t0
    kc = int(nc / 3)
    ref = np.mean(spectra["dns"], axis=0)[: kc]
    err = {}
    for name in ("les", "plain", "fallback"):
        sp = np.mean(spectra[name], axis=0)[: kc]
        d, r = sp[1:], ref[1:]
        err[name] = {
            # energy-weighted: sum_k |E - E_dns| / sum_k E_dns over 1 <= k < k_c
            "rel_l1": float(np.sum(np.abs(d - r)) / np.sum(r)),
            # shape: mean_k |log10(E / E_dns)|, every shell weighted alike
            "mean_abs_log10": float(np.mean(np.abs(np.log10(np.maximum(d, 1e-300) / np.maximum(r, 1e-300))))),
            # the top third of the resolved shells, where the closure acts
            "rel_l1_top_third": float(np.sum(np.abs(d - r)[2 * len(r) // 3:]) / np.sum(r[2 * len(r) // 3:])),
        }
        # energy flux through k (resolved transfers) against the DNS's, 1 <= k < k_c
        fl = np.mean(fluxes[name], axis=0)[1:kc]
        fr = np.mean(fluxes["dns"], axis=0)[1:kc]
        err[name]["flux_rel_l1"] = float(np.sum(np.abs(fl - fr)) / max(np.sum(np.abs(fr)), 1e-300))
    return {
        "dns": {"n": nf, "steps_compared": dns_steps, "gpu_s": t_dns_gpu, "physical_time": T},
        "les": {"n": nc, "steps": les_steps, "gpu_s": t_les_gpu, "gain": t_dns_gpu / t_les_gpu},
        "spectrum_error": err,
        "training": {"snapshots": nsnap, "steps": train_steps, "batch": batch, "data_s": t_data, "train_s": t_train,
                     "loss_first": losses[0], "loss_last": float(np.mean(losses[-20:])),
                     "val_loss": float(np.mean(val)) if val else None},
        "omega": omega, "nu": nu, "hnu": hnu, "total_s": time.perf_counter() - t_all,
    }
