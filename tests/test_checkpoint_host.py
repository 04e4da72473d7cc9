"""Checkpoint formats on the host: the reference's Parameters file round trip (with the
exact layout its parser expects) and the .npz scan state."""
import numpy as np

from ansatzevolve_gb300 import checkpoint


def test_parameters_file_round_trip(tmp_path, golden):
    fx = golden("h4")
    sets = np.asarray(fx["angles"])
    E = np.asarray(fx["E"])
    p = tmp_path / "H4_Parameters.dat"
    checkpoint.write_parameters(p, sets, E)
    text = p.read_text().splitlines()
    assert text[0] == str(sets.shape[1]) and "=" in text[1]
    got, gE = checkpoint.read_parameters(p)
    assert len(got) == len(sets)
    for a, b in zip(got, sets):
        np.testing.assert_allclose(a, b, atol=1e-15, rtol=1e-14)
    np.testing.assert_allclose(gE, E, atol=1e-15, rtol=1e-14)


def test_parameters_energy_line_follows_the_reference_parser(tmp_path):
    """The energy is the number after '=' on the line following the count (the
    reference's fscanf("%*[^=]= %lg %*[^\\n]")), whatever text surrounds it."""
    p = tmp_path / "X_Parameters.dat"
    p.write_text("3\nEnergy of minimum      1=  -2.844887240192929 first found at step 5 after 245 function calls\n"
                 "0.5\n-0.25\n1.0\n")
    sets, E = checkpoint.read_parameters(p)
    assert np.array_equal(sets[0], [0.5, -0.25, 1.0]) and E[0] == -2.844887240192929


def test_scan_state_round_trip(tmp_path):
    s = np.linspace(0, 1, 5)
    x = np.random.default_rng(0).normal(size=(5, 7))
    E = -np.arange(5.0)
    p = tmp_path / "scan.npz"
    checkpoint.save_scan(p, s, x, E, [2024, 77])
    s2, x2, E2, seeds = checkpoint.load_scan(p)
    assert np.array_equal(s, s2) and np.array_equal(x, x2) and np.array_equal(E, E2)
    assert list(seeds) == [2024, 77]
