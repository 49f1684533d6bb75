"""Copy the reference's thermal-conductivity fixtures into tests/golden/ (run once, in a
container that has the reference checkout; the copies travel with the repository).

  python tests/golden/make_golden.py /path/to/tdep

Copied data files (the reference's own test inputs and expected output, unmodified):
  mgo/infile.ucposcar                    tests/infiles/infile.ucposcar
  mgo/infile.forceconstant               tests/infiles/infile.forceconstant        (polar MgO FC2)
  mgo/infile.forceconstant_thirdorder    tests/infiles/infile.forceconstant_thirdorder
  mgo/outfile.thermal_conductivity.ref   tests/thermal_conductivity/reference/outfile.thermal_conductivity
  mgo/outfile.dispersion_relations.ref   tests/phonon_dispersion_relations/reference/outfile.dispersion_relations
A SHA-256 manifest of the sources is written to mgo/MANIFEST.
"""
import hashlib
import shutil
import sys
from pathlib import Path

FILES = {
    "infile.ucposcar": "tests/infiles/infile.ucposcar",
    "infile.forceconstant": "tests/infiles/infile.forceconstant",
    "infile.forceconstant_thirdorder": "tests/infiles/infile.forceconstant_thirdorder",
    "outfile.thermal_conductivity.ref": "tests/thermal_conductivity/reference/outfile.thermal_conductivity",
    "outfile.dispersion_relations.ref": "tests/phonon_dispersion_relations/reference/outfile.dispersion_relations",
}


def main(ref_root: str) -> None:
    root = Path(ref_root)
    out = Path(__file__).resolve().parent / "mgo"
    out.mkdir(exist_ok=True)
    lines = []
    for dst, src in FILES.items():
        shutil.copyfile(root / src, out / dst)
        h = hashlib.sha256((root / src).read_bytes()).hexdigest()
        lines.append(f"{h}  {src}  -> {dst}")
    (out / "MANIFEST").write_text("\n".join(lines) + "\n")
    print("\n".join(lines))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the tdep checkout>")
    main(sys.argv[1])
