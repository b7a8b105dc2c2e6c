"""The oracle against golden fixtures made by the reference's own CUDA kernels.

tests/golden/make_golden.py ran the reference's kernels (compiled from its sources, issued in the
order of its host loop, main.cu:32-85) for 60 steps from seeded starts of the two pin cases and
stored sampled fields, population norms, particle states, solid-node counts, link checksums and the
new-fluid list.  The oracle, run from the same inputs on the CPU, must reproduce them:
fields within 1e-12 relative (the reference is compiled with FMA contraction, the oracle without),
integer structures exactly, link q sums within 1e-10 per link, particle columns within 1e-9 of
their column scale.
"""
import os
import sys

import numpy as np
import pytest

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
import make_golden as MG  # noqa: E402

GOLDEN = os.path.join(REPO, "tests", "golden")


def _field_close(got, ref, scale, tol=1e-12):
    return np.linalg.norm(got - ref) / max(scale, 1e-300) < tol


def check_against_golden(impl, case, data):
    """impl: an object with the oracle's / Solver's accessors, already stepped MG.STEPS steps."""
    nodes, pop_nodes = data["nodes"], data["pop_nodes"]
    f, g = impl.fg()
    L = f.size // 27
    f, g = f.reshape(27, L), g.reshape(27, L)
    gscale = np.linalg.norm(data["g_norm"])
    assert _field_close(np.linalg.norm(g, axis=1), data["g_norm"], gscale)
    assert _field_close(np.linalg.norm(f, axis=1), data["f_norm"], gscale)
    assert _field_close(g[:, pop_nodes], data["g"], np.linalg.norm(data["g"]))
    assert _field_close(f[:, pop_nodes], data["f"], np.linalg.norm(data["g"]))
    m = impl.macros()
    for k, name in enumerate(["rho", "ux", "uy", "uz", "phi", "force_x"]):
        ref = data["macros"][k]
        den = max(np.linalg.norm(ref), 1e-3 * np.linalg.norm(data["macros"][4]))
        assert np.linalg.norm(m[name][nodes] - ref) / den < 1e-12, name
    if "particles" in data:
        npart = len(data["particles"])
        p = impl.particles()
        scale = np.maximum(np.abs(data["particles"]).max(0), 1e-300)
        assert np.all(np.abs(p - data["particles"]).max(0) <= 1e-9 * scale + 1e-15)
        assert np.array_equal(MG.solid_counts(impl.flags(), npart), data["solid"])
        node, d, pid, q = impl.links()
        got = MG.link_checksums(node, d, pid, q, npart)
        ref = data["links"]
        assert np.array_equal(got[:, :3], ref[:, :3])                 # count, sum of nodes and dirs
        assert np.all(np.abs(got[:, 3] - ref[:, 3]) <= 1e-10 * np.maximum(ref[:, 0], 1))
        nf_node, nf_pid = impl.new_fluid()
        ref_nf = data["newfluid"][np.argsort(data["newfluid"][:, 0], kind="stable")]
        assert np.array_equal(nf_node, ref_nf[:, 0]) and np.array_equal(nf_pid, ref_nf[:, 1])


@pytest.mark.parametrize("case", MG.CASES)
def test_oracle_reproduces_reference_kernels(oracle_mod, case):
    data = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    assert int(data["steps"]) == MG.STEPS
    cfg, f, g, f7, parts = MG.inputs(case, oracle_mod)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7, parts)
    if parts is not None:
        npart = len(parts)
        assert np.array_equal(MG.solid_counts(o.flags(), npart), data["solid0"])
        node, d, pid, q = o.links()
        got = MG.link_checksums(node, d, pid, q, npart)
        assert np.array_equal(got[:, :3], data["links0"][:, :3])
        assert np.all(np.abs(got[:, 3] - data["links0"][:, 3]) <= 1e-12 * np.maximum(data["links0"][:, 0], 1))
    o.step(MG.STEPS)
    check_against_golden(o, case, data)
    o.close()
