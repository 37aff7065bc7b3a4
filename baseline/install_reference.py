"""Install GisAPR's own code into baseline/_ref for the reference arm of
bench.py -- BENCH INFRASTRUCTURE, never imported by the package.

    python baseline/install_reference.py --reference <GisAPR source root>

GisAPR is a flat directory of scripts plus two source zips, not a Python
package. The recipe first tries the offline pip install of the reference
the benchmark contract names; that fails for want of a setup.py or
pyproject.toml, so it then unpacks the two trees the reference arm runs,
unmodified, into baseline/_ref/:

* GisAPR-210-optimized/  (GisAPR-210-optimized-3.zip: the v606 search with
  in-memory volumes, pdb2mrc v3, pdb_text) -- the CPU torch path;
* GisAPR-210-DE-v1.3.2/  (GisAPR-Lite-v1.3.2.zip: pdb2mrc v4 and the NVRTC
  ``deposit`` kernel of gisapr_cuda_density.py) -- the GPU splat bar.

baseline/_ref/INSTALL.txt records what happened. The folder is git-ignored;
it travels with the working tree to the machine that runs the benchmark,
where nothing reads the original sources.
"""
from __future__ import annotations

import argparse
import shutil
import subprocess
import sys
import zipfile
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
DEST = ROOT / "baseline" / "_ref"
TREES = {"GisAPR-210-optimized-3.zip": "GisAPR-210-optimized", "GisAPR-Lite-v1.3.2.zip": "GisAPR-210-DE-v1.3.2"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of the GisAPR sources (flat script directory with the two zips)")
    args = ap.parse_args()
    ref = Path(args.reference)
    DEST.mkdir(parents=True, exist_ok=True)
    log = []
    r = subprocess.run([sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation",
                        "--find-links", "/opt/wheelhouse", "--target", str(DEST / "pip"), str(ref)],
                       capture_output=True, text=True)
    tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or [""]
    log.append(f"pip install --target: exit {r.returncode}: {tail[0]}")
    shutil.rmtree(DEST / "pip", ignore_errors=True)
    for zname, tree in TREES.items():
        shutil.rmtree(DEST / tree, ignore_errors=True)
        with zipfile.ZipFile(ref / zname) as z:
            members = [m for m in z.namelist() if m.endswith(".py") or m.endswith(".md") or m.endswith("LICENSE")]
            z.extractall(DEST, members=members)
        log.append(f"unpacked {zname} -> baseline/_ref/{tree} ({len(members)} files)")
    (DEST / "INSTALL.txt").write_text("\n".join(log) + "\n")
    print("\n".join(log))


if __name__ == "__main__":
    main()
