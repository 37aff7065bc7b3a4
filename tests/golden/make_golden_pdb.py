"""Generate the PDB-reader fixture by running GisAPR's reference reader.

    python tests/golden/make_golden_pdb.py --reference <GisAPR source root>

The reference's pdb_text.read_pdb (top-level tree) reads a set of PDB texts
that exercise its rules: MODEL/ENDMDL spans (first model or all models),
HETATM with and without the HETATM switch, explicit element columns, atom
names aligned as one-letter elements, unaligned two-letter names, names
with digits, unknown names, missing chain ids and short lines. For every
text and switch combination the fixture stores the coordinates, elements,
chains and line indices, or the error it raised.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent


def atom(rec, serial, name, res, chain, x, y, z, element=""):
    line = f"{rec:<6}{serial:5d} {name:<4} {res:>3} {chain:1}{1:4d}    {x:8.3f}{y:8.3f}{z:8.3f}{1.0:6.2f}{0.0:6.2f}"
    return line + (f"          {element:>2}" if element else "") + "\n"


def texts():
    base = [
        atom("ATOM", 1, " N  ", "ALA", "A", 1.0, 2.0, 3.0, "N"),
        atom("ATOM", 2, " CA ", "ALA", "A", 1.5, 2.5, 3.5),
        atom("ATOM", 3, "CA  ", "ALA", "A", -1.5, 0.25, 9.125),
        atom("HETATM", 4, "CA  ", "CA", "B", 4.0, 5.0, 6.0),
        atom("HETATM", 5, "FE1 ", "HEM", "B", 7.0, 8.0, 9.0),
        atom("ATOM", 6, "1HB ", "ALA", "A", 0.0, 0.0, 0.0),
        atom("ATOM", 7, "SG  ", "CYS", "A", 3.0, 3.0, 3.0),
        atom("HETATM", 8, "CL  ", "CL", "C", 1.0, 1.0, 1.0),
        atom("HETATM", 9, "ZZ9 ", "UNK", "C", 2.0, 2.0, 2.0),
        atom("ATOM", 10, "OXT ", "ALA", " ", 5.0, 5.0, 5.0, "XX"),
        atom("HETATM", 11, "MG  ", "MG", "D", 6.0, 6.0, 6.0, "Mg"),
        atom("ATOM", 12, " SE ", "MSE", "A", 1.0, 0.0, 0.0),
        atom("HETATM", 13, "SE  ", "MSE", "A", 2.0, 0.0, 0.0),
        atom("ATOM", 14, "'C1 ", "DNA", "E", 3.0, 0.0, 0.0),
        atom("ATOM", 15, "    ", "UNK", "E", 4.0, 0.0, 0.0),
    ]
    plain = "HEADER    TEST\n" + "".join(base) + "TER\nEND\n"
    models = ("REMARK before\n" + atom("ATOM", 90, " C  ", "GLY", "Z", 9.0, 9.0, 9.0) + "MODEL        1\n"
              + "".join(base[:5]) + "ENDMDL\nMODEL        2\n" + "".join(base[5:10]) + "ENDMDL\n"
              + atom("ATOM", 91, " O  ", "GLY", "Z", 8.0, 8.0, 8.0) + "MODEL        3\n" + "".join(base[10:])
              + "ENDMDL\nEND\n")
    no_end = "MODEL        1\n" + "".join(base[:3]) + "MODEL        2\n" + "".join(base[3:6]) + "END\n"
    stray = "ENDMDL\nMODEL        1\n" + "".join(base[:3]) + "ENDMDL\n"
    bad = "".join(base[:2]) + base[2][:30] + "   x.000   1.000   2.000\n"
    nonfinite = "".join(base[:2]) + base[2][:30] + "     nan   1.000   2.000\n"
    return dict(plain=plain, models=models, no_end=no_end, stray=stray, bad=bad, nonfinite=nonfinite)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="root of the GisAPR sources (flat script directory with the two zips)")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    spec = importlib.util.spec_from_file_location("ref_pdb_text", Path(args.reference) / "pdb_text.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ref_pdb_text"] = mod
    spec.loader.exec_module(mod)
    cases = []
    with tempfile.TemporaryDirectory() as td:
        for name, text in texts().items():
            path = Path(td) / f"{name}.pdb"
            path.write_text(text)
            for het in (True, False):
                for first in (True, False):
                    try:
                        p = mod.read_pdb(str(path), include_hetatm=het, first_model_only=first)
                        out = dict(coords=p.coords.astype(float).tolist(), elements=p.elements.tolist(),
                                   chains=p.chains.tolist(), lines=p.atom_line_indices.tolist())
                    except ValueError:
                        out = "error"
                    cases.append(dict(text=name, include_hetatm=het, first_model_only=first, result=out))
    (Path(args.out) / "golden_pdb.json").write_text(json.dumps(dict(texts=texts(), cases=cases), indent=1) + "\n")
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
