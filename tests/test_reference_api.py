"""Host-side mirror of the reference's Parameters (input-file keys, atoi/atof
semantics, defaults) -- CPU only."""
from lbmminiapp_gb300.reference_api import Parameters


def test_parameters_keys_and_defaults(tmp_path):
    p = Parameters()
    assert (p.propPattern, p.pullSetting, p.unrollSetting, p.simulationSize, p.timesteps) == (0, 0, 0, 1.0, 1)
    assert p.omega == 1.0 and p.gravity == 0.000001 and p.lattice == 19
    f = tmp_path / "in.txt"
    f.write_text("# comment\n\nsimulationSize 2.0\npropPattern 1\npull 1\nunroll 1\ndensityChange 0.02\n"
                 "writevtk 0\ntimesteps 250\nunknownKey 7\ntau 0.8\nlattice 27\nstorage f16\n")
    p.readInput(f)
    assert p.getSimulationSize() == 2.0 and p.getPropPattern() == 1 and p.getPullSetting() == 1
    assert p.getUnrollSetting() == 1 and p.densityChange == 0.02 and p.getTimesteps() == 250
    assert abs(p.omega - 1.25) < 1e-15 and p.lattice == 27 and p.storage == "f16"
    assert len(p.echo) == 13


def test_lowercase_aliases_and_atoi(tmp_path):
    f = tmp_path / "in.txt"
    f.write_text("simulationsize 4\nproppattern 1.7\ntimesteps 12.9\ndensitychange 0.5\n")
    p = Parameters().readInput(f)
    assert p.simulationSize == 4.0 and p.propPattern == 1 and p.timesteps == 12 and p.densityChange == 0.5
