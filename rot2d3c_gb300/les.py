"""Learned-closure experiment: DNS -> filtered training data -> CNN -> LES.

1. A fine FP32 run (DNS) on nf^2 with time-constant random-phase forcing in
   the shell 4-6 is spun up and sampled: every ``snap_every`` CFL steps the
   state is filtered onto the coarse nc^2 grid (sharp cutoff k <= nc/3) and
   the 8 network inputs and the 2 subgrid bracket tendencies are stored
   (``r2d3c_closure_sample``), with the filtered energy spectrum and energy
   flux of every snapshot.
2. The closure CNN is trained on random batches with Adam (inputs and targets
   standardised per channel); the last 10% of the snapshots in time are held
   out, and the network's per-shell skill on them is measured (band_fit).
3. From several held-out filtered DNS states (``starts``), the coarse runs
   advance over the same physical time: the LES with the CNN tendencies
   (re-evaluated at every step), the plain coarse solver, and the fallback
   with hyperviscosity (nn > 1).  Their energy spectra and fluxes, averaged
   over the second half of every run and over the starts, are compared with
   the filtered DNS's, averaged over its whole sampled record, for k < k_c;
   the GPU time per unit of physical time of the LES is compared with the
   DNS's.

A network whose held-out loss is not below 0.9 (1 = no better than
predicting the mean) is not applied: that LES runs as the hyperviscous
fallback.

The LES applies the network's tendencies only on the shells next to the
cutoff, 2 k_c/3 <= k <= k_c (``band``, r2d3c_closure_set_band).  The subgrid
transfer of a sharp cutoff acts there; on the large scales the network's
output is mostly error, and as a persistent random forcing of the weakly
damped large scales that error builds a spurious condensate (with the
tendencies on every shell the LES held 2-9 times the DNS energy in shells
1-2 and lost to the hyperviscous fallback in energy-weighted measures).

No counterpart in the reference program.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import DT_CFL, FP32, Context, make_params
from .closure import CNN, band_fit, closure_advance, closure_sample, set_band


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


def spectrum_errors(sp, ref, fl, flr, kc):
    """Errors of a mean energy spectrum ``sp`` and flux ``fl`` against the
    reference ``ref``, ``flr`` over the shells 1 <= k < kc."""
    d, r = np.asarray(sp)[1:kc], np.asarray(ref)[1:kc]
    fl, flr = np.asarray(fl)[1:kc], np.asarray(flr)[1:kc]
    top = 2 * len(r) // 3
    return {
        # energy-weighted: sum_k |E - E_dns| / sum_k E_dns
        "rel_l1": float(np.sum(np.abs(d - r)) / np.sum(r)),
        # shape: mean_k |log10(E / E_dns)|, every shell weighted alike
        "mean_abs_log10": float(np.mean(np.abs(np.log10(np.maximum(d, 1e-300) / np.maximum(r, 1e-300))))),
        # the top third of the resolved shells, where the closure acts
        "rel_l1_top_third": float(np.sum(np.abs(d - r)[top:]) / np.sum(r[top:])),
        # largest relative error of any shell
        "max_shell_rel": float(np.max(np.abs(d - r) / r)),
        # energy flux through k (resolved transfers) against the DNS's
        "flux_rel_l1": float(np.sum(np.abs(fl - flr)) / max(np.sum(np.abs(flr)), 1e-300)),
    }


def band_weights(rule, kc, nb, lsq=None):
    """Per-shell weights of the LES tendencies ([2, nb] float32) for a band
    rule: None (no weighting: every shell), "near_cutoff" (1 on the shells
    2 kc/3 <= k <= kc, 0 elsewhere), ("high", k) (1 on the shells k .. kc),
    or "lsq" (the held-out least-squares weights ``lsq``)."""
    if rule is None:
        return None
    if rule == "lsq":
        return lsq
    if rule == "near_cutoff":
        rule = ("high", 2 * kc // 3)
    if isinstance(rule, (tuple, list)) and rule[0] == "high":
        w = np.zeros((2, nb), np.float32)
        w[:, int(rule[1]):kc + 1] = 1.0
        return w
    raise ValueError(f"unknown band rule {rule!r}")


def _rule_name(rule):
    if rule is None:
        return "les_all_shells"
    if isinstance(rule, str):
        return "les_" + rule
    return f"les_{rule[0]}{rule[1]}"


def _flux(c):
    """Running sum over k of the total energy transfer (2-D part + vz part)."""
    _, f1, f2 = c.transfers()
    return np.cumsum(f1 + f2)


def dns_dataset(nf=2048, nc=256, omega=1.0, nu=2e-5, nsnap=1000, snap_every=10, spinup=2000, cfl=0.5, seed=1,
                hnu=0.1, starts=4):
    """Stage 1: the spun-up DNS and its filtered snapshots -- network inputs
    X and subgrid targets Y (device), the filtered spectrum and the energy
    flux of every snapshot, and the filtered states of ``starts`` held-out
    snapshots (the last 10% in time) as LES initial conditions."""
    import torch
    ps, vz, fp, fz = _setup_run(nf, seed)
    pf = make_params(n=nf, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0,
                     cfl=cfl)
    fine = Context(pf, FP32)
    fine.set_state(ps, vz)
    fine.set_forcing(fp, fz)
    fine.set_time(0.0)
    t_dns, _ = fine.advance(spinup, DT_CFL, cfl)
    pc = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0,
                     cfl=cfl)
    coarse = Context(pc, FP32)
    X = torch.empty((nsnap, nc, nc, 8), dtype=torch.float32, device="cuda")
    Y = torch.empty((nsnap, nc, nc, 2), dtype=torch.float32, device="cuda")
    ntrain = max(1, int(0.9 * nsnap))
    nstart = max(1, min(starts, nsnap - ntrain))
    start_ids = [ntrain + (nsnap - ntrain) * s // nstart for s in range(nstart)]
    start_states, spec, flx, snap_t = {}, [], [], []
    t0 = time.perf_counter()
    for i in range(nsnap):
        t_dns, _ = fine.advance(snap_every, DT_CFL, cfl)
        closure_sample(fine, coarse, X[i], Y[i])
        spec.append(coarse.spectrum()[0])
        flx.append(_flux(fine)[: nc // 2 + 1])
        snap_t.append(t_dns)
        if i in start_ids:
            start_states[i] = coarse.get_state()
    torch.cuda.synchronize()
    return {"fine": fine, "coarse": coarse, "X": X, "Y": Y, "ntrain": ntrain, "start_ids": start_ids,
            "start_states": start_states, "spec": spec, "flux": flx, "snap_t": snap_t, "t_dns": t_dns,
            "forcing": coarse_forcing(fp, fz, nf, nc), "data_s": time.perf_counter() - t0,
            "cfg": dict(nf=nf, nc=nc, omega=omega, nu=nu, hnu=hnu, cfl=cfl, nsnap=nsnap)}


def train_network(ds, train_steps=3000, batch=32, lr=1e-3, seed=1):
    """Stage 2: the CNN trained with Adam on random batches of the first 90%
    of the snapshots (inputs and targets standardised per channel); its
    held-out loss."""
    import torch
    X, Y, ntrain = ds["X"], ds["Y"], ds["ntrain"]
    nsnap, nc = X.shape[0], X.shape[1]
    net = CNN(nc, nc, batch, seed)
    im, isd = X.mean(dim=(0, 1, 2)).cpu().numpy(), X.std(dim=(0, 1, 2)).cpu().numpy()
    om, osd = Y.mean(dim=(0, 1, 2)).cpu().numpy(), Y.std(dim=(0, 1, 2)).cpu().numpy()
    net.set_normalization(im, np.maximum(isd, 1e-12), om, np.maximum(osd, 1e-12))
    bx = torch.empty((batch, nc, nc, 8), dtype=torch.float32, device="cuda")
    by = torch.empty((batch, nc, nc, 2), dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    losses = []
    t0 = time.perf_counter()
    for s in range(train_steps):
        idx = torch.randint(0, ntrain, (batch,), device="cuda", generator=gen)
        torch.index_select(X, 0, idx, out=bx)
        torch.index_select(Y, 0, idx, out=by)
        losses.append(net.train_step(bx, by, batch, lr))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    val = []
    for i in range(ntrain, nsnap, batch):
        b = min(batch, nsnap - i)
        val.append(net.gradients(X[i:i + b].contiguous(), Y[i:i + b].contiguous(), b)[0])
    return net, {"snapshots": nsnap, "steps": train_steps, "batch": batch, "lr": lr, "data_s": ds["data_s"],
                 "train_s": t_train, "loss_first": losses[0], "loss_last": float(np.mean(losses[-20:])),
                 "val_loss": float(np.mean(val)) if val else None}


def evaluate(ds, net, les_steps=4000, spec_every=50, fallback_nn=4, bands=("near_cutoff",), time_dns=True,
             val_loss=None, skill_gate=0.9, every=1, overlap=False):
    """Stage 3: from every held-out start, the plain coarse solver, the
    hyperviscous fallback and one LES per band rule (``bands``, see
    band_weights) advance les_steps CFL steps; spectra and fluxes averaged
    over the second half of every run and over the starts are compared with
    the filtered DNS's over its whole record.  With time_dns, the DNS
    continues over one LES run's mean physical time for the GPU-time gain
    (of the first band rule's LES).  A network whose held-out loss
    ``val_loss`` (standardised: 1 = predicting the mean) is not below
    ``skill_gate`` has no skill to apply: its LES runs as the hyperviscous
    fallback, the closure's stated fallback.  every: the network is
    evaluated before every every-th LES step (its tendencies held between);
    overlap: the network runs one step behind, beside the step
    (closure_advance with overlap)."""
    import torch
    cfg = ds["cfg"]
    nc, nu, hnu, omega, cfl = cfg["nc"], cfg["nu"], cfg["hnu"], cfg["omega"], cfg["cfl"]
    les_steps = max(spec_every, les_steps // spec_every * spec_every)
    kc = int(nc / 3)
    nb = nc // 2 + 1
    lsq = band_fit(net, ds["X"], ds["Y"], range(ds["ntrain"], ds["X"].shape[0]), nc)
    cfp, cfz = ds["forcing"]
    models = {}
    for name, nn_, nuc in (("plain", 1, nu), ("fallback", fallback_nn, None)):
        p = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=nn_, mm=2, nnv=nn_, mmv=2, omega=omega, iflow=0,
                        cfl=cfl)
        if nuc is None:  # hyperviscosity with the same damping rate at the coarse cutoff
            p.nu = p.nuv = nu * kc ** 2 / kc ** (2 * nn_) * 20.0
        models[name] = (p, None)
    pl = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0, cfl=cfl)
    gated = val_loss is not None and not (val_loss < skill_gate)
    les_names = []
    for b in bands:
        models[_rule_name(b)] = (models["fallback"][0], None) if gated else (pl, b)
        les_names.append(_rule_name(b))
    spectra = {k: [] for k in models}
    fluxes = {k: [] for k in models}
    per_start = {k: [] for k in models}
    t_les_gpu = {k: 0.0 for k in les_names}
    T = 0.0
    for name, (p, rule) in models.items():
        c = Context(p, FP32)
        c.set_forcing(cfp, cfz)
        w = band_weights(rule, kc, nb, lsq) if name in les_names else None
        if w is not None:
            set_band(c, w)
        for si in ds["start_ids"]:
            ps_c, vz_c = ds["start_states"][si]
            c.set_state(ps_c, vz_c)
            c.set_time(ds["snap_t"][si])
            sp_run, fl_run = [], []
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            t_end = ds["snap_t"][si]
            for s in range(0, les_steps, spec_every):
                if name in les_names and not gated:
                    t_end, _ = closure_advance(c, net, spec_every, DT_CFL, cfl, every=every, overlap=overlap)
                else:
                    t_end, _ = c.advance(spec_every, DT_CFL, cfl)
                if s + spec_every > les_steps // 2:
                    sp_run.append(c.spectrum()[0])
                    fl_run.append(_flux(c))
            torch.cuda.synchronize()
            if name in les_names:
                t_les_gpu[name] += time.perf_counter() - t0
                if name == les_names[0]:
                    T += t_end - ds["snap_t"][si]
            spectra[name] += sp_run
            fluxes[name] += fl_run
            per_start[name].append((np.mean(sp_run, axis=0), np.mean(fl_run, axis=0)))
        c.destroy()
    nst = len(ds["start_ids"])
    T /= nst
    dns = {"n": cfg["nf"], "physical_time": T,
           "reference": f"filtered DNS spectra and fluxes averaged over all {len(ds['spec'])} snapshots"}
    les = {"n": nc, "steps": les_steps, "starts": nst, "gpu_s": {k: v / nst for k, v in t_les_gpu.items()},
           "note": "gpu_s and physical_time per LES run (mean over starts)",
           "network_applied": not gated,
           "gate": f"held-out loss {val_loss} {'>=' if gated else '<'} {skill_gate}" if val_loss is not None else None}
    if time_dns:
        fine = ds["fine"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        td0 = td = ds["t_dns"]
        dns_steps = 0
        while td < td0 + T:
            td, _ = fine.advance(8, DT_CFL, cfl)
            dns_steps += 8
        torch.cuda.synchronize()
        ds["t_dns"] = td
        dns.update(steps_compared=dns_steps, gpu_s=time.perf_counter() - t0)
        les["gain"] = dns["gpu_s"] / les["gpu_s"][les_names[0]]
    ref = np.mean(ds["spec"], axis=0)
    refl = np.mean(ds["flux"], axis=0)
    err, spread = {}, {}
    for name in models:
        err[name] = spectrum_errors(np.mean(spectra[name], axis=0), ref, np.mean(fluxes[name], axis=0), refl, kc)
        ps_err = [spectrum_errors(a, ref, b, refl, kc) for a, b in per_start[name]]
        spread[name] = {k: [e[k] for e in ps_err] for k in ps_err[0]}
    spectra_mean = {k: np.mean(spectra[k], axis=0)[:kc].tolist() for k in models}
    spectra_mean["dns"] = ref[:kc].tolist()
    return {"dns": dns, "les": les, "spectrum_error": err, "spectrum_error_per_start": spread,
            "skill": {"omega": lsq[0, :kc + 1].round(3).tolist(), "vz": lsq[1, :kc + 1].round(3).tolist(),
                      "definition": "per-shell least-squares weight of the network's output against held-out "
                                    "targets (1: no correction needed, 0: no skill)"},
            "spectra": spectra_mean}


def step_timing(nc=256, steps=200, seed=1, nu=2e-5, hnu=1.0, omega=1.0, cfl=0.5):
    """GPU time per coarse step (CUDA events on the context's stream, graph
    replay after a warm-up) of the plain solver and of the LES with the
    network before every step, before every second step, and one step
    behind beside the step (closure_advance's overlap), at nc^2 with the
    closure experiment's coefficients and band rule and a freshly created
    network (the timing does not depend on its weights).  Returns
    {"plain": us, "every_1": us, "every_2": us, "overlap": us}."""
    import torch
    steps = max(2, steps // 2 * 2)
    ps, vz, fp, fz = _setup_run(nc, seed)
    p = make_params(n=nc, nu=nu, nuv=nu, hnu=hnu, hnuv=hnu, nn=1, mm=2, nnv=1, mmv=2, omega=omega, iflow=0, cfl=cfl)
    c = Context(p, FP32)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    net = CNN(nc, nc, 1, seed)
    set_band(c, band_weights("near_cutoff", nc // 3, nc // 2 + 1))
    st = torch.cuda.ExternalStream(c.stream())
    runs = {"plain": lambda k: c.advance(k, DT_CFL, cfl),
            "every_1": lambda k: closure_advance(c, net, k, DT_CFL, cfl),
            "every_2": lambda k: closure_advance(c, net, k, DT_CFL, cfl, every=2),
            "overlap": lambda k: closure_advance(c, net, k, DT_CFL, cfl, overlap=True)}
    out = {}
    for name, run in runs.items():
        run(10)  # capture and warm-up
        c.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        run(steps)
        e1.record(st)
        e1.synchronize()
        out[name] = 1e3 * e0.elapsed_time(e1) / steps
    net.destroy()
    c.destroy()
    return out


def run_experiment(nf=2048, nc=256, omega=1.0, nu=2e-5, nsnap=1000, snap_every=10, spinup=2000,
                   train_steps=3000, batch=32, lr=1e-3, les_steps=4000, cfl=0.5, seed=1,
                   fallback_nn=4, spec_every=50, hnu=0.1, starts=4, band="near_cutoff", compare_bands=(), every=1,
                   overlap=False):
    """The three stages; returns a dict of timings and errors.

    nf, nc: DNS and LES grids; nu: viscosity of both (nn = 1); omega:
    rotation rate; hnu: large-scale (hypo)viscosity of all runs (mm = 2);
    nsnap snapshots taken every snap_every DNS steps after spinup steps;
    train_steps Adam steps of batch snapshots; ``starts`` coarse runs of
    les_steps CFL steps per model, from held-out snapshots, whose second
    halves are averaged for the spectra (one spectrum every spec_every
    steps); band: the band rule of the LES tendencies (band_weights);
    every: network evaluations every that many LES steps (spec_every must
    be a multiple); overlap: the network one step behind, beside the step;
    compare_bands: further LES band rules run for comparison.  The fallback
    run replaces the viscosity by a hyperviscosity of order fallback_nn with
    the damping rate 20 nu k_c^2 at the cutoff k_c = nc/3.
    """
    t_all = time.perf_counter()
    ds = dns_dataset(nf=nf, nc=nc, omega=omega, nu=nu, nsnap=nsnap, snap_every=snap_every, spinup=spinup, cfl=cfl,
                     seed=seed, hnu=hnu, starts=starts)
    net, training = train_network(ds, train_steps=train_steps, batch=batch, lr=lr, seed=seed)
    ev = evaluate(ds, net, les_steps=les_steps, spec_every=spec_every, fallback_nn=fallback_nn,
                  bands=(band,) + tuple(compare_bands), val_loss=training["val_loss"], every=every,
                  overlap=overlap)
    name = _rule_name(band)
    err = {"les": ev["spectrum_error"][name], "plain": ev["spectrum_error"]["plain"],
           "fallback": ev["spectrum_error"]["fallback"]}
    err.update({k: v for k, v in ev["spectrum_error"].items() if k not in (name, "plain", "fallback")})
    les = dict(ev["les"], gpu_s=ev["les"]["gpu_s"][name], band=band if isinstance(band, (str, type(None)))
               else list(band), network_every=every, network_overlap=overlap)
    ds["fine"].destroy()
    ds["coarse"].destroy()
    net.destroy()
    return {"dns": ev["dns"], "les": les, "spectrum_error": err,
            "spectrum_error_per_start": ev["spectrum_error_per_start"], "skill": ev["skill"],
            "spectra": ev["spectra"], "training": training,
            "omega": omega, "nu": nu, "hnu": hnu, "total_s": time.perf_counter() - t_all}
