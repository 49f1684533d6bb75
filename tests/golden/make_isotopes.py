"""Extract the natural isotope compositions the reference tabulates
(src/libolle/type_crystalstructure.f90, subroutine naturaldistribution) into
tests/golden/isotopes.json, the fixture tests/test_host.py checks the library's own table
against (run once, in a container that has the reference checkout):

  python tests/golden/make_isotopes.py <path of the tdep checkout>

The JSON maps an element symbol to [[abundance, mass in amu], ...] in the file's order.
"""
import json
import re
import sys
from pathlib import Path


def main(ref_root: str) -> None:
    src = (Path(ref_root) / "src/libolle/type_crystalstructure.f90").read_text()
    body = src[src.index("subroutine naturaldistribution"):]
    body = body[: body.index("end subroutine")]
    out = {}
    for m in re.finditer(r'case\("(\w+)"\)(.*?)(?=case\(|end select)', body, re.S):
        sym, blk = m.group(1), m.group(2)
        conc = {int(i): float(v) for i, v in re.findall(r"self%conc\((\d+)\)\s*=\s*([0-9.eEdD+-]+)_flyt", blk)}
        mass = {int(i): float(v) for i, v in re.findall(r"self%mass\((\d+)\)\s*=\s*([0-9.eEdD+-]+)_flyt", blk)}
        if conc and sorted(conc) == sorted(mass):
            out[sym] = [[conc[i], mass[i]] for i in sorted(conc)]
    dst = Path(__file__).resolve().parent / "isotopes.json"
    dst.write_text(json.dumps(out, indent=0, sort_keys=True) + "\n")
    print(f"{len(out)} elements -> {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_isotopes.py <path of the tdep checkout>")
    main(sys.argv[1])
