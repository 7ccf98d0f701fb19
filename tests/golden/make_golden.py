"""Records outputs of the reference's own kernel as golden fixtures.

Run on a GPU host with the reference cubin built (oracle/_ref/):

    python tests/golden/make_golden.py OUTDIR

For each case it writes OUTDIR/<name>.npz (catalogues cat0.., and `hist`, the
reference's triCountsAll_) and OUTDIR/<name>.json (box, edges, survey flag,
which catalogue plays p1/p2/p3, weighted flag; for the rppi bin type also
the number of pi bins and the weight written past the histogram's end). The
committed copies in
tests/golden/ pin the CPU oracle in tests/test_oracle.py, where no GPU is
available. Inputs are the seeded cases of tests/cases.py, trimmed to keep the
fixtures small.
"""
import json
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tests import cases  # noqa: E402


def all_cases():
    out = []
    for make in cases.KATS:
        c = make()
        out.append((make.__name__, c["box"], c["edges"], c["survey"], [c["p"]], [0, 0, 0], (0, 0, 0)))
    c = cases.fma_probe()
    out.append(("fma_probe", c["box"], c["edges"], False, [c["p"]], [0, 0, 0], (0, 0, 0)))
    for name, make, n in [("box_uniform", cases.small_box_uniform, 2000),
                          ("box_clustered", cases.small_box_clustered, 2500),
                          ("box_nondivisible", cases.small_box_nondivisible, 2500),
                          ("box_tiny_grid", cases.small_box_tiny_grid, 600),
                          ("box_one_cell", cases.small_box_one_cell, 60)]:
        p, box, edges = make()
        out.append((name, box, edges, False, [np.ascontiguousarray(p[:n])], [0, 0, 0], (0, 0, 0)))
    for weighted in (False, True):
        d, r, box, ori, edges = cases.small_survey(nd=1000, nr=2000, weighted=weighted)
        tag = "survey_ddr_weighted" if weighted else "survey_ddr"
        out.append((tag, box, edges, True, [d, r], [0, 0, 1], ori))
        if not weighted:
            out.append(("survey_drr", box, edges, True, [d, r], [0, 1, 1], ori))
    return out


def all_rppi_cases():
    """(name, box, edges, npi, survey, catalogues, roles, ori) of the rppi fixtures."""
    out = []
    for make in cases.RPPI_KATS:
        c = make()
        out.append((make.__name__, c["box"], c["edges"], c["npi"], False, [c["p"]], [0, 0, 0], (0, 0, 0)))
    for name, make in [("rppi_box_probe", cases.rppi_box_probe), ("rppi_survey_probe", cases.rppi_survey_probe)]:
        c = make()
        out.append((name, c["box"], c["edges"], c["npi"], c["survey"], [c["p"]], [0, 0, 0], c["ori"]))
    for name, make, n in [("rppi_box_uniform", cases.rppi_small_box, 1500),
                          ("rppi_box_clustered", cases.rppi_small_box_clustered, 1500),
                          ("rppi_box_nondivisible", cases.rppi_small_box_nondivisible, 1200)]:
        p, box, edges, npi = make()
        out.append((name, box, edges, npi, False, [np.ascontiguousarray(p[:n])], [0, 0, 0], (0, 0, 0)))
    for weighted in (False, True):
        d, r, box, ori, edges, npi = cases.rppi_small_survey(nd=800, nr=1600, weighted=weighted)
        tag = "rppi_survey_ddr_weighted" if weighted else "rppi_survey_ddr"
        out.append((tag, box, edges, npi, True, [d, r], [0, 0, 1], ori))
        if not weighted:
            out.append(("rppi_survey_ddd", box, edges, npi, True, [d, r], [0, 0, 0], ori))
    return out


def main(outdir: str) -> None:
    od = pathlib.Path(outdir)
    od.mkdir(parents=True, exist_ok=True)
    O.runner()
    for name, box, edges, survey, cats, roles, ori in all_cases():
        args = [cats[i] for i in roles]
        hist, kms, tms = O.reference_count(box, edges, *args, survey=survey, ori=ori)
        weighted = any(bool(np.any(c[:, 3] != 1.0)) for c in cats)
        np.savez_compressed(od / f"{name}.npz", hist=hist, **{f"cat{i}": c for i, c in enumerate(cats)})
        meta = {"box": float(np.broadcast_to(box, (3,))[0]) if np.ndim(box) == 0 else list(map(float, box)),
                "edges": list(map(float, edges)), "survey": bool(survey),
                "roles": [f"cat{i}" for i in roles], "weighted": weighted,
                "ori": list(map(float, ori)), "sizes": [int(len(c)) for c in cats],
                "reference_kernel_ms": kms, "triangles": float(hist.sum()),
                "source": "reference source/device.cu kernels via oracle/ref_runner.cu"}
        (od / f"{name}.json").write_text(json.dumps(meta, indent=1) + "\n")
        print(f"{name}: sum={hist.sum():.0f} kernel {kms:.2f} ms")
    for name, box, edges, npi, survey, cats, roles, ori in all_rppi_cases():
        args = [cats[i] for i in roles]
        hist, overflow, kms, tms = O.reference_count_rppi(box, edges, npi, *args, survey=survey, ori=ori)
        weighted = any(bool(np.any(c[:, 3] != 1.0)) for c in cats)
        np.savez_compressed(od / f"{name}.npz", hist=hist, **{f"cat{i}": c for i, c in enumerate(cats)})
        meta = {"box": list(map(float, np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))),
                "edges": list(map(float, edges)), "num_pi_bins": int(npi), "survey": bool(survey),
                "roles": [f"cat{i}" for i in roles], "weighted": weighted,
                "ori": list(map(float, ori)), "sizes": [int(len(c)) for c in cats],
                "overflow": float(overflow), "reference_kernel_ms": kms, "triangles": float(hist.sum()),
                "source": "reference source/device.cu rppi kernels via oracle/ref_runner.cu"}
        (od / f"{name}.json").write_text(json.dumps(meta, indent=1) + "\n")
        print(f"{name}: sum={hist.sum():.0f} overflow={overflow} kernel {kms:.2f} ms")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py OUTPUT_DIR")
    main(sys.argv[1])
