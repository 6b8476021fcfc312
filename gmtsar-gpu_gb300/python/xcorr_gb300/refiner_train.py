"""Training data and training loop of the subpixel refiner.

Training windows come from the plain correlation path itself: synthetic
images made of independent 256 x 256 speckle tiles, each with its own
(slave) shift -- a random integer part in [-4, 4] px plus a subpixel part
uniform in [-0.5, 0.5] px in each axis -- and its own SNR, uniform in
0..30 dB.  One window sits on each tile (128x128 windows, 256x256 patches,
as the 128^2-window configuration), with range interpolation 2 (the
reference's default, refiner/subpix_refiner.f32) or 1 (no range
interpolation: the surrogate form, refiner/subpix_refiner_ri1.f32).  The plain
path returns each window's normalised 9x9 peak neighbourhood (the refiner's
input) and its integer offset; the target is the subpixel position of the
true peak in surface pixels, fx = xoff - ri*dx, fy = yoff - dy, the
quantities highres_corr estimates as xfrac/yfrac.

Every network computation (forward, backward, Adam, inference) runs in the
library's CUDA kernels; torch only supplies device memory and the random
tiles.

    python -m xcorr_gb300.refiner_train --windows 2000000 [--ri 1] --out <dir>
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

import xcorr_gb300 as xg

TILE = 256
HERE = os.path.dirname(os.path.abspath(__file__))
REFINER_DIR = os.path.join(os.path.dirname(os.path.dirname(HERE)), "refiner")
DEFAULT_WEIGHTS = os.path.join(REFINER_DIR, "subpix_refiner.f32")


def weights_name(ri: int) -> str:
    """File name of the trained parameters for surfaces of range interpolation ri."""
    return "subpix_refiner.f32" if ri == 2 else f"subpix_refiner_ri{ri}.f32"


def weights_path(ri: int) -> str:
    return os.path.join(REFINER_DIR, weights_name(ri))


def load_weights(path: str = DEFAULT_WEIGHTS) -> np.ndarray:
    w = np.fromfile(path, dtype="<f4")
    if w.size != xg.REFINER_NPARAM:
        raise ValueError(f"{path}: {w.size} values, expected {xg.REFINER_NPARAM}")
    return w


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases, log-variance bias -4 (float32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in (("W1", (32, 9)), ("b1", (32,)), ("W2", (32, 288)), ("b2", (32,)), ("W3", (32, 288)),
                        ("b3", (32,)), ("F1", (64, 288)), ("c1", (64,)), ("F2", (3, 64)), ("c2", (3,))):
        if name[0] in "WF":
            a = rng.standard_normal(shape) * math.sqrt(2.0 / shape[1])
            if name == "F2":
                a *= 0.1
        else:
            a = np.zeros(shape)
            if name == "c2":
                a[2] = -4.0
        parts.append(a.ravel())
    return np.concatenate(parts).astype(np.float32)


def make_tiles(ntx: int, nty: int, seed: int, device):
    """Master/slave int16 images of ntx x nty independent tiles (torch, on
    `device`), the tile-centre locations and each tile's true shift."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    B = ntx * nty
    m = torch.randn((B, TILE, TILE, 2), generator=g, device=device).mul_(1000.0).round_().clamp_(-32768, 32767)
    frac = torch.rand((B, 2), generator=g, device=device, dtype=torch.float64) - 0.5
    intg = torch.randint(-4, 5, (B, 2), generator=g, device=device).to(torch.float64)
    shift = frac + intg                                         # (dx, dy)
    snr = torch.rand((B,), generator=g, device=device, dtype=torch.float64) * 30.0
    nfrac = torch.pow(10.0, -snr / 10.0)
    k = torch.fft.fftfreq(TILE, device=device, dtype=torch.float64)
    mz = torch.complex(m[..., 0], m[..., 1]).to(torch.complex128)
    ramp = torch.exp(-2j * math.pi * (k[None, :, None] * shift[:, 1, None, None] + k[None, None, :] * shift[:, 0, None, None]))
    sz = torch.fft.ifft2(torch.fft.fft2(mz) * ramp)
    nz = torch.randn((B, TILE, TILE, 2), generator=g, device=device, dtype=torch.float64) * (1000.0 * torch.sqrt(nfrac))[:, None, None, None]
    s = torch.stack([sz.real, sz.imag], dim=-1) + nz
    s = s.round_().clamp_(-32768, 32767)
    def to_image(t):
        t = t.to(torch.int16).reshape(nty, ntx, TILE, TILE, 2).permute(0, 2, 1, 3, 4)
        return t.reshape(nty * TILE, ntx * TILE, 2).contiguous()
    ty, tx = np.meshgrid(np.arange(nty), np.arange(ntx), indexing="ij")
    locs = np.stack([tx.ravel() * TILE + TILE // 2, ty.ravel() * TILE + TILE // 2], axis=1).astype(np.int32)
    return to_image(m), to_image(s), locs, shift.cpu().numpy(), snr.cpu().numpy()


def plain_windows(ctx, master, slave, locs, device):
    """Plain path on one tile image: results (numpy) and 9x9 neighbourhoods (torch)."""
    import torch
    n = len(locs)
    feat = torch.zeros((n, 81), dtype=torch.float32, device=device)
    res = torch.zeros((n, xg.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=device)
    dl = torch.from_numpy(locs).to(device)
    ctx.set_features(feat.data_ptr())
    ny, nx = master.shape[0], master.shape[1]
    ctx.correlate_device(master.data_ptr(), nx, ny, slave.data_ptr(), nx, ny, dl.data_ptr(), n, res.data_ptr(),
                         torch.cuda.current_stream(device).cuda_stream)
    ctx.set_features(None)
    torch.cuda.synchronize(device)
    r = np.frombuffer(res.cpu().numpy().tobytes(), dtype=xg.RESULT_DTYPE)
    return r, feat


def targets(r, shift, ri):
    fx = r["xoff"].astype(np.float64) - ri * shift[:, 0]
    fy = r["yoff"].astype(np.float64) - shift[:, 1]
    return np.stack([fx, fy], axis=1).astype(np.float32)


def dataset(nwin: int, seed: int, device, tiles_side: int = 32, ri: int = 2):
    """nwin training windows: features (torch), targets (torch), plain results, shifts."""
    import torch
    ctx = xg.Context(xg.params(TILE // 4, TILE // 4, ri, 1, 16), device=device.index)
    feats, tgts, plains, shifts, snrs = [], [], [], [], []
    per = tiles_side * tiles_side
    for i in range((nwin + per - 1) // per):
        m, s, locs, sh, snr = make_tiles(tiles_side, tiles_side, seed * 100003 + i, device)
        r, f = plain_windows(ctx, m, s, locs, device)
        feats.append(f)
        tgts.append(torch.from_numpy(targets(r, sh, ri)).to(device))
        plains.append(r)
        shifts.append(sh)
        snrs.append(snr)
    ctx.close()
    return (torch.cat(feats)[:nwin], torch.cat(tgts)[:nwin], np.concatenate(plains)[:nwin],
            np.concatenate(shifts)[:nwin], np.concatenate(snrs)[:nwin])


def evaluate(ref, feat, tgt, plain, device, max_sigma=0.15, max_dis=0.25, ri=2):
    """Errors of the refiner, of the plain FFT interpolation and of the combined
    rule (refiner where confident, plain elsewhere), in original pixels (the
    range axis divided by the range interpolation factor), on windows whose
    integer peak is within one pixel of the truth: against the truth, and
    against the plain method's own output (the FP64 oracle's result up to
    FP32 near-ties)."""
    import torch
    n = feat.shape[0]
    out = torch.zeros((n, 3), dtype=torch.float32, device=device)
    ref.forward(feat.data_ptr(), n, out.data_ptr(), tensor_cores=True)
    torch.cuda.synchronize(device)
    o = out.cpu().numpy().astype(np.float64)
    t = tgt.cpu().numpy().astype(np.float64)
    f = feat.cpu().numpy()
    pl = np.stack([plain["xfrac"], plain["yfrac"]], axis=1).astype(np.float64)
    good = (np.abs(t[:, 0]) < 1.0) & (np.abs(t[:, 1]) < 1.0)

    def vertex(a, b, c):
        den = a - 2 * b + c
        return np.where(den < 0, 0.5 * (a - c) / np.where(den < 0, den, -1), 0.0)
    px = vertex(f[:, 39], f[:, 40], f[:, 41])
    py = vertex(f[:, 31], f[:, 40], f[:, 49])
    sg = np.exp(0.5 * o[:, 2])
    use = (sg < max_sigma) & (np.abs(o[:, 0] - px) < max_dis) & (np.abs(o[:, 1] - py) < max_dis) & (f[:, 40] > 0)
    mix = np.where(use[:, None], o[:, :2], pl)

    def rms(a, b):
        d = (a - b)[good]
        return dict(x=float(np.sqrt(np.mean((d[:, 0] / ri) ** 2))), y=float(np.sqrt(np.mean(d[:, 1] ** 2))))
    return dict(windows=int(n), range_interp=ri, within_one_px=int(good.sum()), refiner_used=float(use[good].mean()),
                sigma_quantiles=[float(q) for q in np.quantile(sg[good], [0.1, 0.5, 0.9])],
                max_sigma=max_sigma, max_disagree=max_dis,
                rms_vs_truth_px=dict(refiner=rms(o[:, :2], t), fft_interp=rms(pl, t), combined=rms(mix, t)),
                rms_vs_plain_px=dict(refiner=rms(o[:, :2], pl), combined=rms(mix, pl)))


def train(nwin: int, steps_per_epoch: int | None = None, epochs: int = 12, batch: int = 4096, lr: float = 2e-3,
          seed: int = 1, device=None, log=print, target: str = "truth", ri: int = 2):
    """target "truth": the generator's shift; "plain": the plain method's own
    subpixel answer (the network then stands in for the FFT interpolation)."""
    import torch
    device = device or torch.device("cuda", 0)
    t0 = time.time()
    feat, tgt, plain, shift, snr = dataset(nwin, seed, device, ri=ri)
    hold = max(4096, nwin // 20)
    if target == "plain":
        import torch as _t
        tgt_train = _t.from_numpy(np.stack([plain["xfrac"], plain["yfrac"]], axis=1).astype(np.float32)).to(device)
    else:
        tgt_train = tgt
    ftr, ttr = feat[hold:], tgt_train[hold:]
    fte, tte, pte = feat[:hold], tgt[:hold], plain[:hold]
    # windows whose integer peak is off by more than a pixel carry no subpixel information
    keep = (ttr.abs() < 1.0).all(dim=1)
    ftr, ttr = ftr[keep].contiguous(), ttr[keep].contiguous()
    log(f"data: {nwin} windows ({len(ftr)} kept for training, {hold} held out) in {time.time() - t0:.1f} s")
    ref = xg.Refiner(device.index, max_batch=batch)
    ref.set_params(init_params(seed))
    ntr = len(ftr)
    spe = steps_per_epoch or max(1, ntr // batch)
    g = torch.Generator(device=device).manual_seed(seed)
    t1 = time.time()
    step = 0
    total = epochs * spe
    for ep in range(epochs):
        perm = torch.randperm(ntr, generator=g, device=device)
        for i in range(spe):
            idx = perm[(i * batch) % max(1, ntr - batch):][:batch]
            fb, tb = ftr[idx].contiguous(), ttr[idx].contiguous()
            cur = lr * 0.5 * (1 + math.cos(math.pi * step / total))      # cosine decay
            ref.train_step(fb.data_ptr(), tb.data_ptr(), len(idx), cur)
            step += 1
        loss, _, _ = ref.gradient(fte[:batch].contiguous().data_ptr(), tte[:batch].contiguous().data_ptr(), min(batch, hold))
        log(f"epoch {ep + 1}/{epochs}: held-out loss {loss:.4f}")
    torch.cuda.synchronize(device)
    train_s = time.time() - t1
    report = evaluate(ref, fte, tte, pte, device, ri=ri)
    report.update(train_windows=int(ntr), steps=step, batch=batch, train_seconds=train_s,
                  data_seconds=t1 - t0, seed=seed, target=target, epochs=epochs)
    return ref, report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--windows", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--out", default=os.path.dirname(DEFAULT_WEIGHTS))
    ap.add_argument("--target", default="truth", choices=["truth", "plain"])
    ap.add_argument("--ri", type=int, default=2, choices=[1, 2], help="range interpolation of the surfaces")
    a = ap.parse_args()
    ref, report = train(a.windows, epochs=a.epochs, target=a.target, ri=a.ri)
    os.makedirs(a.out, exist_ok=True)
    ref.get_params().astype("<f4").tofile(os.path.join(a.out, weights_name(a.ri)))
    rep_name = "train_report.json" if a.ri == 2 else f"train_report_ri{a.ri}.json"
    with open(os.path.join(a.out, rep_name), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report, indent=1))


if __name__ == "__main__":
    main()
