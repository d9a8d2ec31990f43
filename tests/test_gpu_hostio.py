"""Large host transfers: results read back into pageable arrays (through the
library's page-locked staging ring, several chunks) are bit-identical to the
same results read into page-locked arrays, and a basis uploaded from pageable
memory (ring + copy threads) gives bit-identical spectra to the same basis
uploaded from page-locked memory (direct copies overlapping the transposes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system(synth):
    # 833 MB of coefficients (13 ring chunks pageable, 4 device chunks
    # page-locked); chi0 after KK is 91 x 91 x 1000 complex = 132 MB
    return synth.build(synth.config_grid24(nbnd=30, nocc=8, npw=1500, nlf=91, lf="xyz", no=1001))


def test_pageable_and_pagelocked_transfers_agree(system, rpa):
    torch = pytest.importorskip("torch")
    s = system
    pinned = torch.empty(s.coeff.shape, dtype=torch.complex128, pin_memory=True).numpy()
    pinned[...] = s.coeff
    outs = []
    for src in (s.coeff, pinned):
        ctx = rpa.Context(precision=rpa.PREC_MIXED)
        ctx.set_gvectors(s.miller, s.G, s.KC)
        ctx.load_basis(s.npw, s.igk, src, s.E)
        ctx.kmap(s.ktot, s.K1, s.R1, s.K2, s.R2, s.iG0)
        ctx.set_q(s.q, s.ilf, s.parG)
        S0, _ = ctx.chi0(rpa.MODE_CHARGE, **rpa.sloss_args(s))
        chi_pageable = ctx.kk(rpa.KK_SLOSS_REAL)
        chi_pinned = torch.empty(chi_pageable.shape, dtype=torch.complex128, pin_memory=True).numpy()
        ctx.kk(rpa.KK_SLOSS_REAL, out=chi_pinned)
        assert np.array_equal(chi_pageable, chi_pinned)
        assert np.isfinite(chi_pageable).all() and np.abs(chi_pageable).max() > 0
        outs.append((S0, chi_pageable))
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
