"""File output of the main sampling (MCI::storeObservablesOnFile / storeWalkerPositionsOnFile,
src/MCIntegrator.cpp:495-542): the reference's line format, every freq-th step of chain 0,
and the observable columns equal to the observables of the recorded walker (an
accumulator prints the values of its last accumulation, here nskip 3)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_observable_and_walker_files(tmp_path):
    import mcintegratorplusplus_gb300 as mcig
    g = mcig.MCI(3, 4, precision=mcig.PREC_FP64)
    g.setSeed(5)
    g.addSamplingFunction(mcig.PDF_GAUSS)
    g.setNdecorrelationSteps(200)
    g.addObservable(mcig.OBS_X2SUM, (), 0, 1, False, mcig.EST_NOOP)
    g.addObservable(mcig.OBS_XND, (), 0, 3, False, mcig.EST_NOOP)
    fo, fw = tmp_path / "observables.txt", tmp_path / "walker.txt"
    g.storeObservablesOnFile(fo, 100)
    g.storeWalkerPositionsOnFile(fw, 50)
    g.integrate(1000)
    wl = fw.read_text().splitlines()
    ol = fo.read_text().splitlines()
    assert len(wl) == 20 and len(ol) == 10
    assert all("   " in line for line in wl) and all(line.endswith(" ") for line in ol)
    walker = {int(line.split()[0]): np.array(line.split()[1:], dtype=float) for line in wl}
    assert sorted(walker) == list(range(0, 1000, 50))
    for line in ol:
        f = line.split()
        r, vals = int(f[0]), np.array(f[1:], dtype=float)
        assert r % 100 == 0 and vals.size == 4
        np.testing.assert_allclose(vals[0], (walker[r] ** 2).sum(), rtol=2e-5)       # x.x at step r
        if (r - r % 3) in walker:                                                     # x_i of step r - r % 3
            np.testing.assert_allclose(vals[1:], walker[r - r % 3], rtol=2e-5, atol=1e-5)
    # cleared files are not written again
    g.clearObservableFile()
    g.clearWalkerFile()
    fo.unlink()
    g.integrate(300)
    assert not fo.exists()
    with pytest.raises(ValueError):
        g.storeObservablesOnFile(fo, 0)
