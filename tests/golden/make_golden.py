"""Writes the golden fixtures tests/golden/<case>.npz.

Cases in tests/cases.CASES are run by the UNMODIFIED serial reference
(oracle/_ref/libserialref.so, built from mate-szoke/ParallelLbmCranfield
serial/ by ``make -C oracle ref``) on the generated mesh written to files in
the reference format.  Cases in cases.ORACLE_ONLY (behaviour the reference
does not have) are produced by the C restatement (oracle/_build) and marked
``source = port``.

Each fixture keeps the per-step residual lines, the sums and sums of squares
of rho/u/v over all cells, the full state of a fixed sample of cells, and
the port's FP64 full-field diagnostics.

    python tests/golden/make_golden.py            # all cases
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
import cases  # noqa: E402


def run_case(name, spec, params, start, steps, use_ref):
    mesh = cases.build_mesh(spec)
    op = cases.oracle_params(params)
    st = cases.start_state(mesh, params, start)
    port = O.Port(mesh.nodes, mesh.conns, **op)
    if st is not None:
        port.set_state(*st)
    _, presid = port.run(steps)
    pstate = port.state()
    diag = port.diagnostics()
    source = "port"
    resid, state = presid, pstate
    if use_ref:
        with tempfile.TemporaryDirectory() as td:
            nf, cf = os.path.join(td, "D2node.dat"), os.path.join(td, "BCconnectors.dat")
            mesh.write(nf, cf)
            ref = O.Ref(nf, cf, op["uavg"], op["vavg"], op["rho_ini"], op["viscosity"],
                        op["inlet_profile"], op["model"], op["curved"], op["outlet"],
                        op["drag_id"])
            if st is not None:
                ref.set_state(*st)
            _, resid = ref.run(steps)
            state = ref.state()
            ref.close()
        source = "reference"
        for k in state:
            if not np.array_equal(state[k], pstate[k]):
                raise SystemExit(f"{name}: port differs from the reference in {k}")
        if not np.array_equal(resid, presid):
            raise SystemExit(f"{name}: port residuals differ from the reference")
    idx = cases.sample_cells(mesh)
    out = dict(source=np.array(source), steps=np.array(steps), resid=resid, sample=idx,
               diag=diag)
    for k in ("rho", "u", "v"):
        out[f"sum_{k}"] = np.array([state[k].sum(), (state[k] ** 2).sum()])
        out[f"s_{k}"] = state[k][idx]
    out["s_F"] = state["F"][idx]
    out["s_METAF"] = state["METAF"][idx]
    out["s_drag"] = state["drag"][idx]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: {source}, {steps} steps, mass {state['rho'].sum():.12g}")


def main():
    O.build()
    use_ref = O.ref_available()
    if not use_ref:
        raise SystemExit("the reference harness is not built (needs the reference sources)")
    for name, (spec, params, start, steps) in cases.CASES.items():
        run_case(name, spec, params, start, steps, True)
    for name, (spec, params, start, steps) in cases.ORACLE_ONLY.items():
        run_case(name, spec, params, start, steps, False)


if __name__ == "__main__":
    main()
