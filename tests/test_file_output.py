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


def test_files_equal_the_references_own_files_byte_for_byte(tmp_path):
    """The reference's own observable and walker files of a main sampling run (recorded by
    oracle/ref_recorder.cpp into tests/golden/reference_golden.json), against the device's files
    of the same run in FP64 replay: the draws are the reference's (the oracle records them;
    it reproduces the reference's engine and distributions bit for bit), so every line must
    be identical, byte for byte."""
    import mcintegratorplusplus_gb300 as mcig
    from oracle import oracle as orc
    import cases

    g = cases.golden()
    fc = g["file_case"]

    def configure(m):
        m.add_sampling_function(mcig.PDF_GAUSS)
        m.set_nfind_mrt2_iterations(-50)
        m.set_ndecorrelation_steps(fc["ndecorr"])
        m.add_observable(mcig.OBS_X2SUM, (), 0, 1, False, mcig.EST_NOOP)
        m.add_observable(mcig.OBS_XND, (), 0, 3, False, mcig.EST_NOOP)

    o = orc.OracleMCI(3, 1)
    o.set_seeds([fc["seed"]])
    configure(o)
    o.set_record(True)
    o.integrate(0, True, True)
    o.integrate(fc["nmc"], False, False)
    tape, lens = o.get_tapes()
    d = mcig.MCI(3, 1, precision=mcig.PREC_FP64)
    configure(d)
    d.setReplay(tape, lens)
    d.integrate(0, True, True)
    fo, fw = tmp_path / "observables.txt", tmp_path / "walker.txt"
    d.storeObservablesOnFile(fo, fc["obs_freq"])
    d.storeWalkerPositionsOnFile(fw, fc["wlk_freq"])
    d.integrate(fc["nmc"], False, False)
    assert fw.read_text() == g["file_wlk"]
    assert fo.read_text() == g["file_obs"]
