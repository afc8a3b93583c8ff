"""Two-site observables, energy and spin read-out after a full anneal, GPU against the FP64
oracle on the same configs (the reference computes no two-site quantity; the oracle defines
<Z_u Z_v> as the BP two-site contraction and the energy as sum J <ZZ> + sum h <Z>).

complex128 kernels: <Z_u Z_v> within 1e-8, energy within 1e-9 relative, sign read-out
identical wherever |<Z>| > 1e-6.  complex64 kernels (measured over these cases: <Z_u Z_v>
3.8e-5, energy 1.6e-6 relative): <Z_u Z_v> within 1e-4, energy within 1e-5 relative, read-out
identical wherever |<Z>| > 1e-3.
"""
import numpy as np
import pytest

from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from bqa_gb300.engine import Annealer  # noqa: E402
from bqa_gb300.layout import build_context  # noqa: E402
from oracle import bqa_oracle as orc  # noqa: E402

CASES = ["tree9", "rr3_n16_chi4", "rr3_n24_chi8", "mixed_n18_chi3", "rr4_n20_chi4", "grid3x4_chi4_damped"]


def _oracle(conf):
    octx = orc.make_context(dict(conf))
    st = orc.initialize_state(octx)
    for ins in octx.instructions:
        if isinstance(ins, dict):
            orc.run_layer(octx, ins["xtime"], ins["ztime"], st)
    z = orc.bloch_vectors(orc.get_density_matrices(octx, st))[:, 2]
    zz = orc.edge_zz(octx, st)
    return z, zz, orc.energy(octx, zz, z)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["double", "single"])
def test_observables_match_oracle(name, precision):
    conf = gc.config(name)
    z_w, zz_w, e_w = _oracle(conf)
    ctx = build_context(dict(conf))
    job = Annealer(ctx, precision=precision)
    for ins in ctx.instructions:
        if isinstance(ins, dict):
            job.run_layer(ins["xtime"], ins["ztime"])
    z = job.bloch_vectors()[:, 2]
    zz = job.edge_zz()
    e = job.energy(zz, z)
    spins, spins_w = job.spin_readout(z), np.where(z_w > 0, 1, -1)
    zz_err = float(np.abs(zz - zz_w).max())
    e_rel = abs(e - e_w) / max(abs(e_w), 1e-12)
    print(f"{name} {precision}: <ZZ> max error {zz_err:.2e}, energy rel error {e_rel:.2e}")
    if precision == "double":
        assert zz_err < 1e-8 and e_rel < 1e-9
        sure = np.abs(z_w) > 1e-6
    else:
        assert zz_err < 1e-4 and e_rel < 1e-5
        sure = np.abs(z_w) > 1e-3
    assert np.array_equal(spins[sure], spins_w[sure])
