"""Particle stack preparation on the GPU (read_star_shift_crop_and_generate_new_star_v5.py).

Before a search, the reference re-centres every particle by its STAR origin
(integer pixels, zero fill), crops the centred window and optionally
whitens (divides the spectrum by its radial mean amplitude, then removes a
least-squares plane and normalises to zero mean and unit sigma) and
high-pass filters it, writing new stacks and a new STAR (v5:135-277). Here a
whole chunk of particles goes through one batched float64 pipeline on the
device (csrc/ingest.cu: load + crop, cuFFT Z2Z, radial-bin divide,
normalise, mask multiply); the functions of the reference's module keep
their names and take one image or a stack:

* ``translation_twoD_image(image, trans_X, trans_Y)`` (v5:9-29) -- host;
* ``getSpectrum_divideBySpectrum(img)``, ``normalize(img)``,
  ``highpassfilter(img, high_pass, angpix)`` (v5:42-134) -- device;
* ``preprocess_stack(images, shifts, crop_size, whitening, highpass, ...)``
  -- the per-particle body of the reference's loop (v5:202-235) for a stack;
* ``run_preprocess(args)`` with ``create_gridsearch_parser`` -- the command.

Outputs are float32, as the reference writes its stacks.
"""
from __future__ import annotations

import argparse
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import _native as nat

__all__ = ["translation_twoD_image", "getSpectrum_divideBySpectrum", "normalize", "highpassfilter",
           "preprocess_stack", "create_gridsearch_parser", "run_preprocess", "radial_bins", "highpass_mask"]

SPECTRUM, NORMALIZE, HIGHPASS = 1, 2, 4


def translation_twoD_image(image, trans_X, trans_Y):
    """Shift by round-half-up integer pixels with zero fill (v5:9-29)."""
    tx, ty = int(np.floor(trans_X + 0.5)), int(np.floor(trans_Y + 0.5))
    ys, xs = image.shape
    out = np.zeros_like(image)
    out[max(0, ty):(ys if ty >= 0 else ys + ty), max(0, tx):(xs if tx >= 0 else xs + tx)] = \
        image[max(0, -ty):ys - max(0, ty), max(0, -tx):xs - max(0, tx)]
    return out


def radial_bins(h: int, w: int) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """CSR of the pixels of the unshifted h x w transform grid per bin
    round(radius on the centred grid), and the pixel count of each bin."""
    j, i = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    dist = np.round(np.sqrt((j - h // 2) ** 2 + (i - w // 2) ** 2)).astype(np.int64)
    dist = np.fft.ifftshift(dist)  # bin of every unshifted pixel
    flat = dist.ravel()
    order = np.argsort(flat, kind="stable").astype(np.int32)
    count = np.bincount(flat, minlength=int(flat.max()) + 1)
    ptr = np.zeros(len(count) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(count)
    return ptr, order, count.astype(np.float64)


def highpass_mask(h: int, w: int, high_pass: float, angpix: float) -> np.ndarray:
    """Raised-cosine high-pass of width 4 shells at ``high_pass`` Angstrom,
    in unshifted order (v5:107-134)."""
    ori = h
    ires = round((ori * angpix) / high_pass)
    half = 4 / 2
    low = max(0.0, (ires - half) / ori)
    high = min(w, (ires + half) / ori)
    width = high - low
    y = np.arange(h) - h // 2
    x = np.arange(w) - w // 2
    yy, xx = np.meshgrid(y, x, indexing="ij")
    r = np.sqrt(xx ** 2 + yy ** 2) / ori
    mask = np.ones((h, w), dtype=np.float64)
    mask[r < low] = 0.0
    band = (r >= low) & (r <= high)
    with np.errstate(divide="ignore", invalid="ignore"):
        mask[band] *= 0.5 - 0.5 * np.cos(np.pi * (r[band] - low) / width)
    return np.ascontiguousarray(np.fft.ifftshift(mask))


class _Tables:
    """Device tables per (h, w) (bins) and per (h, w, high_pass, angpix) (masks)."""

    def __init__(self):
        self.bins: Dict[tuple, tuple] = {}
        self.masks: Dict[tuple, torch.Tensor] = {}

    def get_bins(self, h, w, dev):
        key = (h, w, str(dev))
        if key not in self.bins:
            ptr, pix, cnt = radial_bins(h, w)
            self.bins[key] = (torch.from_numpy(ptr).to(dev), torch.from_numpy(pix).to(dev),
                              torch.from_numpy(cnt).to(dev), len(cnt))
        return self.bins[key]

    def get_mask(self, h, w, high_pass, angpix, dev):
        key = (h, w, float(high_pass), float(angpix), str(dev))
        if key not in self.masks:
            self.masks[key] = torch.from_numpy(highpass_mask(h, w, high_pass, angpix)).to(dev)
        return self.masks[key]


_TABLES = _Tables()


def _device(device):
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type != "cuda":
        raise ValueError("particle preparation runs on a CUDA device")
    return dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())


def preprocess_stack(images, shifts=None, crop_size: int = 0, whitening: bool = False, highpass: bool = False,
                     highpass_freq: float = 50.0, angpix: float = 1.0, device=None, flags: Optional[int] = None,
                     chunk: int = 4096) -> torch.Tensor:
    """Shift, crop, whiten and high-pass a stack of particle images.

    ``images``: [n, h, w] (or [h, w]) float array or tensor; ``shifts``:
    [n, 2] (x, y) pixel shifts (rounded half up, as the reference does) or
    None; ``crop_size`` > 0 crops the centred crop_size square. Returns the
    float32 result [n, c, c] on the device. ``flags`` overrides the
    whitening/high-pass switches with the kernel's step bits."""
    dev = _device(device if device is not None else (images.device if torch.is_tensor(images)
                                                     and images.is_cuda else None))
    single = False
    imgs = images if torch.is_tensor(images) else torch.from_numpy(np.ascontiguousarray(images, np.float32))
    if imgs.ndim == 2:
        imgs, single = imgs[None], True
    if imgs.ndim != 3:
        raise ValueError("images must be [n, h, w] or [h, w]")
    n, h, w = (int(v) for v in imgs.shape)
    ch, cw = (int(crop_size), int(crop_size)) if crop_size and crop_size > 0 else (h, w)
    if ch > h or cw > w:
        raise ValueError(f"crop size {crop_size} exceeds the image size {h}x{w}")
    if flags is None:
        flags = (SPECTRUM | NORMALIZE if whitening else 0) | (HIGHPASS if highpass else 0)
    sh = None
    if shifts is not None:
        s = np.asarray(shifts, dtype=np.float64).reshape(-1, 2)
        if len(s) != n:
            raise ValueError("shifts need one (x, y) pair per image")
        sh = torch.from_numpy(np.floor(s + 0.5).astype(np.int32)).to(dev)
    bins = _TABLES.get_bins(ch, cw, dev) if flags & SPECTRUM else (None, None, None, 0)
    mask = _TABLES.get_mask(ch, cw, highpass_freq, angpix, dev) if flags & HIGHPASS else None
    out = torch.empty((n, ch, cw), dtype=torch.float32, device=dev)
    ctx = nat.Context.for_device(dev).handle
    st = nat.stream_of(dev)
    step = max(1, int(chunk))
    work = torch.empty((min(n, step) * ch * cw * 2,), dtype=torch.float64, device=dev) if n else None
    for a in range(0, n, step):
        b = min(n, a + step)
        src = imgs[a:b].to(dev, torch.float32).contiguous()
        nat.call("gisapr_ingest_stack", ctx, st, nat.ptr(src), b - a, h, w,
                 None if sh is None else nat.c_ptr_offset(sh, a * 8), ch, cw, int(flags), nat.ptr(bins[0]),
                 nat.ptr(bins[1]), nat.ptr(bins[2]), int(bins[3]), nat.ptr(mask), nat.ptr(work),
                 nat.c_ptr_offset(out, a * ch * cw * 4))
    return out[0] if single else out


def getSpectrum_divideBySpectrum(img, device=None) -> torch.Tensor:
    """Image(s) with the spectrum divided by its radial mean amplitude (v5:42-59)."""
    return preprocess_stack(img, device=device, flags=SPECTRUM)


def normalize(img, device=None) -> torch.Tensor:
    """Least-squares plane removed, then zero mean and unit sigma (v5:61-106)."""
    return preprocess_stack(img, device=device, flags=NORMALIZE)


def highpassfilter(img, high_pass, angpix, device=None) -> torch.Tensor:
    """Raised-cosine high-pass at ``high_pass`` Angstrom (v5:107-134)."""
    return preprocess_stack(img, device=device, flags=HIGHPASS, highpass_freq=high_pass, angpix=angpix)


# ---------------------------------------------------------------------------
# the command (v5:30-41, 135-277)
# ---------------------------------------------------------------------------


def create_gridsearch_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(description="Crop block images from particle images. The star file should be "
                                            "the output of relion-BBR or relion-SIRM")
    p.add_argument("--star_name", type=str, required=True, help="Input star file")
    p.add_argument("--output_root_name", type=str, default="output")
    p.add_argument("--newboxsize", type=int, default=128)
    p.add_argument("--batchsize", type=int, default=5000)
    p.add_argument("--dohighpass", action="store_true")
    p.add_argument("--highpassFreq", type=float, default=50.)
    p.add_argument("--dowhitening", action="store_true")
    p.add_argument("--doSkipShifting", action="store_true")
    p.add_argument("--doOnlyMakeStar", action="store_true")
    p.add_argument("--gpuid", type=int, default=0)
    return p


def _star_blocks(lines: List[str]):
    """Loops of a STAR file: (labels -> column, header end, data line indices)."""
    from .tables import find_star_table
    parts = find_star_table(lines, ["_rlnImageName"])
    try:
        optics = find_star_table(lines, ["_rlnImagePixelSize"])
    except ValueError:
        optics = None
    return parts, optics


def _set_token(line: str, index: int, value: str) -> str:
    toks = line.split()
    toks[index] = value
    return "\t".join(toks) + "\n"


def run_preprocess(args) -> Dict[str, object]:
    """Write ``<root>_NNNN.mrcs`` stacks of ``batchsize`` prepared particles
    and ``<root>.star`` (the input with new image names, zeroed origins and
    the optics image size), as the reference's command does. Unreadable
    particles are skipped and left out of the new STAR."""
    from .mrc import read_mrc, write_mrc
    from .tables import read_text_lines
    lines = read_text_lines(args.star_name)
    parts, optics = _star_blocks(lines)
    lab = parts.columns
    ii = lab["_rlnImageName"]
    ox, oy = lab.get("_rlnOriginXAngst", -1), lab.get("_rlnOriginYAngst", -1)
    if optics is None:
        raise ValueError("the STAR file has no optics loop with _rlnImagePixelSize")
    opt_rows = list(optics.row_lines)
    pixel = float(optics.tokens(opt_rows[0])[optics.columns["_rlnImagePixelSize"]])
    rows = list(parts.row_lines)
    names = [parts.tokens(r)[ii] for r in rows]
    root = args.output_root_name + "_"
    crop = int(args.newboxsize)
    bs = max(1, int(args.batchsize))
    new_names: List[str] = []
    valid: List[int] = []
    h = w = -1
    if not args.doOnlyMakeStar:
        dev = torch.device(f"cuda:{int(args.gpuid)}")
        cache: Dict[str, np.ndarray] = {}
        batch_imgs: List[np.ndarray] = []
        batch_shift: List[Tuple[float, float]] = []
        batch_index = 1

        def flush():
            nonlocal batch_imgs, batch_shift, batch_index
            if not batch_imgs:
                return
            stack = np.stack(batch_imgs)
            shifts = None if args.doSkipShifting else np.asarray(batch_shift)
            out = preprocess_stack(stack, shifts, crop if crop > 0 else 0, bool(args.dowhitening),
                                   bool(args.dohighpass), float(args.highpassFreq), pixel, device=dev)
            write_mrc(f"{root}{batch_index:04d}.mrcs", out.cpu().numpy(), pixel)
            batch_imgs, batch_shift = [], []
            batch_index += 1

        for k, (r, name) in enumerate(zip(rows, names)):
            try:
                serial, fname = name.split("@", 1)
                if fname not in cache:
                    cache.clear()
                    cache[fname] = read_mrc(fname, mmap=True)
                data = cache[fname]
                img = np.asarray(data[int(serial) - 1] if data.ndim == 3 else data, dtype=np.float32)
                if img.ndim != 2 or img.size == 0:
                    continue
                if h < 0:
                    h, w = img.shape
                if img.shape != (h, w) or (crop > 0 and (crop > h or crop > w)):
                    continue
                toks = parts.tokens(r)
                sx = float(toks[ox]) / pixel if ox >= 0 else 0.0
                sy = float(toks[oy]) / pixel if oy >= 0 else 0.0
            except Exception as exc:  # noqa: BLE001 - the reference skips any unreadable particle
                print(f"Skip failed image: {name}, error: {exc}")
                continue
            batch_imgs.append(img)
            batch_shift.append((sx, sy))
            new_names.append(f"{len(batch_imgs)}@{root}{batch_index:04d}.mrcs")
            valid.append(k)
            if len(batch_imgs) == bs:
                flush()
        flush()
    else:
        for k in range(len(rows)):
            new_names.append(f"{k % bs + 1}@{root}{k // bs + 1:04d}.mrcs")
            valid.append(k)
    # new STAR: the input's lines with the particle rows rewritten
    keep = {rows[k]: new_names[j] for j, k in enumerate(valid)}
    part_rows = set(rows)
    out_lines = []
    size = crop if crop > 0 else h
    for i, line in enumerate(lines):
        if i in part_rows:
            if i not in keep:
                continue
            line = _set_token(line, ii, keep[i])
            if not args.doSkipShifting:
                if ox >= 0:
                    line = _set_token(line, ox, "0.0")
                if oy >= 0:
                    line = _set_token(line, oy, "0.0")
        elif i in opt_rows and "_rlnImageSize" in optics.columns and size > 0:
            line = _set_token(line, optics.columns["_rlnImageSize"], str(size))
        out_lines.append(line if line.endswith("\n") else line + "\n")
    star_out = args.output_root_name + ".star"
    with open(star_out, "w") as fh:
        fh.writelines(out_lines)
    return dict(particles=len(valid), star=star_out, stacks=sorted({n.split("@", 1)[1] for n in new_names}))

