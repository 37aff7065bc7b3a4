"""Generate the golden fixtures by running GisAPR's reference code itself.

Run in a checkout that has the reference sources (they are read, never
modified):

    python tests/golden/make_golden.py --reference <GisAPR source root>

The reference's optimized-3 tree (GisAPR-210-optimized-3.zip, whose v606
accepts an in-memory volume) is extracted to a temporary directory and
imported with a stub ``mrcfile`` module (file IO is bypassed: volumes and
particle images are passed as tensors, exactly as the reference's in-memory
worker does). Each fixture stores the seeded inputs and the reference's
float32 outputs of every stage of one candidate evaluation:

* golden_box32.npz  -- box 32, every stage for all 48 directions and 24
  particles (inputs stored in full);
* golden_box64.npz  -- box 64 / 1.5 A / 200 particles / HEALPix order 2 /
  +-15 deg / psi 15 deg / +-4 px (the CPU-sized published configuration);
  particle images are regenerated from the seed, so the file stores input
  checksums and the outputs: a density slab and checksum, 8 templates,
  4 particles' spectra, per-particle results and the candidate score.
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile
import types
import zipfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from gisapr_gb300 import synthetic as syn  # noqa: E402


def _import_reference(reference: Path, workdir: Path):
    stub = types.ModuleType("mrcfile")

    def _no_io(*a, **k):
        raise RuntimeError("file IO is bypassed while making fixtures")

    stub.mmap = stub.new = stub.open = _no_io
    stub.mrcfile = types.SimpleNamespace(MrcFile=object)
    sys.modules["mrcfile"] = stub
    with zipfile.ZipFile(reference / "GisAPR-210-optimized-3.zip") as z:
        z.extractall(workdir)
    tree = workdir / "GisAPR-210-optimized"
    sys.path.insert(0, str(tree))
    import importlib
    v606 = importlib.import_module(
        "test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_optimized_standalone")
    pdb2mrc = importlib.import_module("pdb2mrc_gpu_ver_fp32_v3")
    pdb_text = importlib.import_module("pdb_text")
    return v606, pdb2mrc, pdb_text


def _write_angle_star(path, rot, tilt):
    with open(path, "w") as f:
        f.write("\ndata_\n\nloop_\n_rlnAngleRot #1\n_rlnAngleTilt #2\n_rlnAnglePsi #3\n")
        for r, t in zip(rot, tilt):
            f.write(f"{float(r)!r}\t{float(t)!r}\t0.0\n")


def _write_particle_star(path, rec):
    with open(path, "w") as f:
        header = ("\ndata_\n\nloop_\n_rlnImageName #1\n_rlnAngleRot #2\n_rlnAngleTilt #3\n"
                  "_rlnAnglePsi #4\n_rlnDefocusU #5\n_rlnDefocusV #6\n_rlnDefocusAngle #7\n")
        f.write(header)
        lines = header.count("\n")
        assert int(rec.line_index[0]) >= lines
        for i in range(len(rec.rot)):
            while lines < int(rec.line_index[i]):
                f.write("\n")
                lines += 1
            vals = [float(v[i]) for v in (rec.rot, rec.tilt, rec.psi, rec.defocus_u,
                                          rec.defocus_v, rec.defocus_angle)]
            f.write(f"{i + 1}@stack.mrcs\t" + "\t".join(repr(v) for v in vals) + "\n")
            lines += 1


def run_reference(v606, pdb2mrc, pdb_text, job: syn.SearchJob, pose, tmp: Path, keep_dirs=None):
    """One candidate evaluation through the reference's own functions, in the
    order of its run_search loop (v606:1594-1825)."""
    import torch
    spec = job.spec
    n, nb = spec.box, spec.new_box
    pdb_path = tmp / "model.pdb"
    pdb_path.write_text(job.model.pdb_text)
    first = pdb_text.read_pdb(str(pdb_path))
    moved = pdb_text.transform_chain_coordinates(first, "A", pose)
    coords, elements = pdb_text.transformed_density_atoms(str(pdb_path), "A", pose, False)
    density = pdb2mrc.generate_volume(str(pdb_path), n, spec.apix, spec.res, device="cpu",
                                      source_pdb=str(pdb_path), chain_id="A", pose=list(pose))
    fixed_sel = first.chains != "A"
    numbers, _ = pdb2mrc.atoms_to_atomic_numbers_and_masses(first.elements)
    fixed_density = pdb2mrc.density_from_coords(first.coords[fixed_sel], numbers[fixed_sel],
                                                n, spec.apix, spec.res, device="cpu")

    ang_path = tmp / "angles.star"
    _write_angle_star(ang_path, job.model_rot, job.model_tilt)
    angles = v606.read_model_angles(str(ang_path))
    star_path = tmp / "particles.star"
    _write_particle_star(star_path, job.records)
    table = v606.read_particle_table(str(star_path))
    records = table.records
    dev = torch.device("cpu")
    layout = v606.PackedFourierLayout(nb, spec.crop, dev)
    new_apix = n / nb * spec.apix
    trans_scale = spec.apix / new_apix
    local = {e[0]: e[1:] for e in v606.build_local_orientation_entries(
        records, angles.rot, angles.tilt, spec.local_range)}
    mask_np = v606.generate_soft_mask((n, n), spec.mask_radius, spec.mask_edge)
    mask = torch.from_numpy(mask_np)
    fsc_path = ""
    if spec.fsc_half_res is not None:
        fsc_path = str(tmp / "fsc.txt")
        with open(fsc_path, "w") as f:
            for k, v in enumerate(job.fsc):
                f.write(f"{k} {float(v)!r}\n")
    fsc_centered = v606.read_fsc_map(fsc_path, n, nb, False)
    packed_fsc = layout.centered_full_to_packed(torch.from_numpy(fsc_centered))
    projector = v606.IntegratedProjector(dev, n, nb, layout, mask, packed_fsc, 8)
    templates = projector.build_templates(density, angles)

    psi_meta = {}
    uniq = {}
    for rec in records:
        fake, eff = v606.psi_sampling_for_record(rec.psi, spec.psi_step, True, spec.local_range)
        psi_meta[rec.line_index] = (fake, eff)
        for a in eff:
            uniq[float(np.round(a, 6))] = None
    bank = v606.PsiGridBank(n, dev, list(uniq.keys()), 8)
    prep = v606.ParticleFourierPreparer(n, nb, dev, layout, mask, bank)
    ctfgen = v606.PackedCTFTorch(nb, new_apix, spec.cs, spec.voltage, spec.kk, dev)
    ctf = ctfgen.batch(records, table.has_ctf)
    ctf_np = v606.PackedCTFNumPy(nb, new_apix, spec.cs, spec.voltage, spec.kk).batch(records, True)
    ws = v606.CorrelationWorkspace(dev)
    out = dict(spectra=[], scores=[], ys=[], xs=[], local_ptr=[0], local_idx=[],
               z=[], peak=[], best_dir=[], best_psi=[], shift_x=[], shift_y=[], angdist=[],
               fake_psi=[], eff_psi=[], l3=[], accu=[])
    raw = []
    for i, rec in enumerate(records):
        idx = local.get(rec.line_index, [])
        fake, eff = psi_meta[rec.line_index]
        out["fake_psi"].append(fake)
        out["eff_psi"].append(eff)
        out["local_idx"].extend(idx)
        out["local_ptr"].append(len(out["local_idx"]))
        image = torch.from_numpy(job.images[i])
        p = prep.prepare(image, eff, ctf[i])
        out["spectra"].append(p.numpy())
        if not idx:
            continue
        lt = templates.index_select(0, torch.tensor(idx, dtype=torch.long))
        s, y, x = v606.correlate_templates_and_particle(lt, p, layout, ws)
        out["scores"].append(s.numpy().copy().ravel())
        out["ys"].append(y.numpy().copy().ravel())
        out["xs"].append(x.numpy().copy().ravel())
        rr = v606.make_result_records(rec, fake, angles.rot, angles.tilt, idx, s, y, x,
                                      layout.crop_size, trans_scale)
        cc, psi_r, raw_r = rr
        out["z"].append(cc[2])
        out["l3"].append(cc[3])
        out["accu"].append(cc[4])
        out["angdist"].append(cc[7])
        out["shift_x"].append(cc[8])
        out["shift_y"].append(cc[9])
        out["best_psi"].append(psi_r[2])
        out["peak"].append(raw_r[2])
        k = int(torch.argmax(s.reshape(-1)).item())
        out["best_dir"].append(idx[k // s.shape[1]])
        raw.append(raw_r[2])
    score = float(np.sum(np.exp(np.asarray(raw, dtype=np.float64) / 1024.0)))
    return dict(
        moved_float=np.asarray(moved, dtype=np.float64),
        density_coords=np.asarray(coords, dtype=np.float32),
        density=density.numpy(), fixed_density=fixed_density.numpy(),
        rot_t=angles.rotation_matrices_t, templates=templates.numpy(),
        ctf=ctf.numpy(), ctf_numpy=ctf_np, mask=mask_np, packed_fsc=packed_fsc.numpy(),
        score=score, **out)


def _flat(lists, dtype):
    return np.asarray([v for l in lists for v in l], dtype=dtype)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    import torch
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        v606, pdb2mrc, pdb_text = _import_reference(Path(args.reference), td / "ref")

        # ---- box 32: everything stored
        spec = syn.WORKLOADS["box32_tiny"]
        job = syn.make_job(spec, seed=11)
        pose = syn.candidate_poses(1, 12, 3.0, 1.5, exact=True)[0]
        r = run_reference(v606, pdb2mrc, pdb_text, job, pose, td)
        rec = job.records
        np.savez_compressed(
            Path(args.out) / "golden_box32.npz",
            spec_name=np.asarray(spec.name), pdb_text=np.asarray(job.model.pdb_text),
            pose=pose, images=job.images, model_rot=np.asarray(job.model_rot),
            model_tilt=np.asarray(job.model_tilt), fsc=job.fsc,
            rec_line=rec.line_index, rec_rot=rec.rot, rec_tilt=rec.tilt, rec_psi=rec.psi,
            rec_dfu=rec.defocus_u, rec_dfv=rec.defocus_v, rec_dfa=rec.defocus_angle,
            moved_float=r["moved_float"], density_coords=r["density_coords"],
            density=r["density"], fixed_density=r["fixed_density"], rot_t=r["rot_t"],
            templates=r["templates"], ctf=r["ctf"], ctf_numpy=r["ctf_numpy"], mask=r["mask"],
            packed_fsc=r["packed_fsc"], spectra=np.stack(r["spectra"]),
            scores=_flat(r["scores"], np.float32), ys=_flat(r["ys"], np.int64),
            xs=_flat(r["xs"], np.int64), local_ptr=np.asarray(r["local_ptr"], np.int64),
            local_idx=np.asarray(r["local_idx"], np.int64),
            fake_psi=np.asarray(r["fake_psi"]), eff_psi=np.asarray(r["eff_psi"]),
            z=np.asarray(r["z"]), peak=np.asarray(r["peak"]), best_dir=np.asarray(r["best_dir"]),
            best_psi=np.asarray(r["best_psi"]), shift_x=np.asarray(r["shift_x"]),
            shift_y=np.asarray(r["shift_y"]), angdist=np.asarray(r["angdist"]),
            l3=np.asarray(r["l3"]), accu=np.asarray(r["accu"]), score=np.asarray(r["score"]))
        print("box32 score", r["score"])

        # ---- box 64, 200 particles: outputs only, inputs regenerated from the seed
        spec = syn.WORKLOADS["box64_200p"]
        job = syn.make_job(spec, seed=21)
        pose = syn.candidate_poses(1, 22, 3.0, 1.5, exact=True)[0]
        r = run_reference(v606, pdb2mrc, pdb_text, job, pose, td)
        sel_t = np.linspace(0, len(job.model_rot) - 1, 8).astype(np.int64)
        sel_p = np.asarray([0, 1, 2, 3], np.int64)
        np.savez_compressed(
            Path(args.out) / "golden_box64.npz",
            spec_name=np.asarray(spec.name), seed=np.asarray(21), pose=pose,
            image_checksum=np.asarray([job.images.astype(np.float64).sum(),
                                       (job.images.astype(np.float64) ** 2).sum()]),
            image_probe=job.images[:, 32, 32].copy(),
            density_slab=r["density"][28:36].copy(),
            density_checksum=np.asarray([r["density"].astype(np.float64).sum(),
                                         (r["density"].astype(np.float64) ** 2).sum()]),
            template_index=sel_t, templates=r["templates"][sel_t],
            particle_index=sel_p, spectra=np.stack(r["spectra"])[sel_p],
            local_ptr=np.asarray(r["local_ptr"], np.int64),
            local_idx=np.asarray(r["local_idx"], np.int64),
            scores=_flat(r["scores"], np.float32), ys=_flat(r["ys"], np.int64),
            xs=_flat(r["xs"], np.int64),
            z=np.asarray(r["z"]), peak=np.asarray(r["peak"]), best_dir=np.asarray(r["best_dir"]),
            best_psi=np.asarray(r["best_psi"]), shift_x=np.asarray(r["shift_x"]),
            shift_y=np.asarray(r["shift_y"]), score=np.asarray(r["score"]))
        print("box64 score", r["score"])


if __name__ == "__main__":
    main()
