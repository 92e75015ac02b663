"""Generate tests/golden/reference_inputs.json from the reference's own test
inputs (its Testin/in/*.in namelist files).

    python tests/golden/make_reference_inputs.py [TESTIN_DIR]

TESTIN_DIR defaults to /root/reference/Testin/in.  Each input is read with
molsim_gb300.reference_input.system_from_input (seed 1 for the positions of
particles that the input places at random; lattices are placed as the
reference's SetLattice places them).  The fixture stores, per input, the
resulting system as plain data (species, types, positions, box, cutoffs,
Ewald and list settings, bonds and angles), the method and time step, or the
reason the input was refused (the variable outside the path).  The GPU tests
(tests/test_gpu_reference_inputs.py) run the stored systems without the
reference's files; tests/test_cpu_reference_input.py checks that the files,
where present, still give the stored systems.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from molsim_gb300 import reference_input  # noqa: E402

OUT = os.path.join(HERE, "reference_inputs.json")
TESTIN = "/root/reference/Testin/in"
INPUTS = ["salt.mc.ew.in", "chain.bd.nohs.in", "chain.md.nohs.in", "lj.md.in", "lj.mc.celllist.in",
          "pe.md.ew.in", "holm.ew1.in", "qq.ew.surf.in", "qq.ew.nosurf.in", "mic.mc.ewspm.in",
          "wnemo.md.ewspm.in"]


def entry(path):
    name = os.path.basename(path)
    try:
        run = reference_input.system_from_input(path, seed=1)
    except (NotImplementedError, ValueError) as ex:
        return {"input": name, "refused": f"{type(ex).__name__}: {ex}"}
    return {"input": name, "method": run.method, "tstep": run.tstep, "iseed": run.iseed,
            "system": run.system.to_dict()}


def make(testin=TESTIN):
    return [entry(os.path.join(testin, f)) for f in INPUTS]


def main():
    testin = sys.argv[1] if len(sys.argv) > 1 else TESTIN
    with open(OUT, "w") as fh:
        json.dump(make(testin), fh, separators=(",", ":"))
    print(OUT)


if __name__ == "__main__":
    main()
