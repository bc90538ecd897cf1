"""Seeded atmospheres of the batched workload, converted by the reference.

Test/bench infrastructure, run in a container that has the reference at
``/root/reference``.  Draws atmospheres with the batched workload's
distributions -- layers uniform in 64..80, Teff log-uniform in 3500..40000 K,
log g uniform in 0..5, [M/H] uniform in -2..+0.5 -- writes each as an ATLAS
``.atm`` grey model (:mod:`kurucz_py_joss_submission_gb300.workloads`),
converts it with the reference's own ``convert_atm_to_npz.py`` and keeps the
fields the synthesis path reads (``atm_batch_<k>.npz``).  A draw the
converter rejects is recorded and skipped.  ``batch_atmospheres.json``
lists what was kept.

Usage: ``python tests/golden/make_batch_atmospheres.py [count]`` (default 8)
"""

from __future__ import annotations

import json
import math
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE))

import make_golden as MG  # noqa: E402
from kurucz_py_joss_submission_gb300 import workloads  # noqa: E402

SEED = 303


def draw(rng):
    return dict(n_layers=int(rng.integers(64, 81)),
                teff=float(math.exp(rng.uniform(math.log(3500.0), math.log(40000.0)))),
                logg=float(rng.uniform(0.0, 5.0)),
                metallicity=float(rng.uniform(-2.0, 0.5)))


def main(argv):
    count = int(argv[0]) if argv else 8
    rng = np.random.default_rng(SEED)
    kept, rejected = [], []
    with tempfile.TemporaryDirectory(prefix="kbatch_") as tmp:
        work = Path(tmp)
        k = 0
        while len(kept) < count and k < 4 * count:
            spec = draw(rng)
            k += 1
            atm = work / f"b{k}.atm"
            workloads.grey_atmosphere_atm(atm, spec["teff"], spec["logg"], spec["metallicity"],
                                          n_layers=spec["n_layers"])
            full = work / f"b{k}.npz"
            r = subprocess.run(
                [sys.executable, str(MG.REFERENCE / "synthe_py/tools/convert_atm_to_npz.py"), str(atm),
                 str(full), "--atlas-tables", str(MG.REFERENCE / "synthe_py/data/atlas_tables.npz")],
                env=MG._env(), cwd=work, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
            if r.returncode != 0 or not full.exists():
                rejected.append(dict(spec, reason=r.stderr.strip().splitlines()[-1:]))
                continue
            with np.load(full) as d:
                out = {f: np.asarray(d[f]) for f in MG.ATM_FIELDS if f in d}
            name = f"atm_batch_{len(kept)}.npz"
            np.savez_compressed(HERE / name, **out)
            kept.append(dict(spec, file=name))
            print("kept", name, spec, flush=True)
    (HERE / "batch_atmospheres.json").write_text(json.dumps(dict(seed=SEED, kept=kept, rejected=rejected),
                                                            indent=1))
    return 0


if __name__ == "__main__":
    raise SystemExit(main(sys.argv[1:]))
