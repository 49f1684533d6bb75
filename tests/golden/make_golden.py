"""Copy the reference's thermal-conductivity fixtures into tests/golden/ (run once, in a
container that has the reference checkout; the copies travel with the repository).

  python tests/golden/make_golden.py /path/to/tdep

Copied data files (the reference's own test inputs and expected output, unmodified):
  mgo/infile.ucposcar                    tests/infiles/infile.ucposcar
  mgo/infile.forceconstant               tests/infiles/infile.forceconstant        (polar MgO FC2)
  mgo/infile.forceconstant_thirdorder    tests/infiles/infile.forceconstant_thirdorder
  mgo/outfile.thermal_conductivity.ref   tests/thermal_conductivity/reference/outfile.thermal_conductivity
  mgo/outfile.dispersion_relations.ref   tests/phonon_dispersion_relations/reference/outfile.dispersion_relations
  hdf5/lineshape_self_energy.hdf5        tests/lineshape/reference/outfile.phonon_self_energy.hdf5
  hdf5/cumulative_kappa_2023.hdf5        tests/thermal_conductivity_2023/reference/outfile.cumulative_kappa.hdf5
(the two HDF5 files are libhdf5-written fixtures for the tests' HDF5 reader). A SHA-256
manifest of the sources is written to mgo/MANIFEST and hdf5/MANIFEST.
"""
import hashlib
import shutil
import sys
from pathlib import Path

FILES = {
    "hdf5/lineshape_self_energy.hdf5": "tests/lineshape/reference/outfile.phonon_self_energy.hdf5",
    "hdf5/cumulative_kappa_2023.hdf5": "tests/thermal_conductivity_2023/reference/outfile.cumulative_kappa.hdf5",
    "infile.ucposcar": "tests/infiles/infile.ucposcar",
    "infile.forceconstant": "tests/infiles/infile.forceconstant",
    "infile.forceconstant_thirdorder": "tests/infiles/infile.forceconstant_thirdorder",
    "outfile.thermal_conductivity.ref": "tests/thermal_conductivity/reference/outfile.thermal_conductivity",
    "outfile.dispersion_relations.ref": "tests/phonon_dispersion_relations/reference/outfile.dispersion_relations",
}


def main(ref_root: str) -> None:
    root = Path(ref_root)
    here = Path(__file__).resolve().parent
    manifests = {}
    for dst, src in FILES.items():
        sub, name = (dst.split("/", 1) if "/" in dst else ("mgo", dst))
        out = here / sub
        out.mkdir(exist_ok=True)
        target = out / name
        if target.exists():
            target.chmod(0o644)
        shutil.copyfile(root / src, target)
        h = hashlib.sha256((root / src).read_bytes()).hexdigest()
        manifests.setdefault(sub, []).append(f"{h}  {src}  -> {name}")
    for sub, lines in manifests.items():
        (here / sub / "MANIFEST").write_text("\n".join(lines) + "\n")
        print("\n".join(lines))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the tdep checkout>")
    main(sys.argv[1])
