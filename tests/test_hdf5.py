"""The HDF5 module and the reference's observable/checkpoint layout (CPU only)."""
import glob
import os

import numpy as np
import pytest


def test_reads_a_libhdf5_file(pkg):
    """A file written by libhdf5 itself (MATLAB v7.3, superblock v0 behind a 512-byte user block)."""
    from pffrg_gb300 import hdf5 as H

    scipy = pytest.importorskip("scipy")
    hits = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data",
                                  "testhdf5_7.4_GLNX86.mat"))
    if not hits:
        pytest.skip("no libhdf5-written test file in this scipy")
    with H.File(hits[0], "r") as f:
        assert f.keys() == ["testdouble"]
        x = f.read("testdouble")
    assert np.allclose(x.ravel(), np.arange(9) * np.pi / 4)


def test_round_trip_types_and_appends(pkg, tmp_path):
    from pffrg_gb300 import hdf5 as H

    p = str(tmp_path / "t_obs")
    rng = np.random.default_rng(0)
    q3 = np.asfortranarray(rng.normal(size=(6, 16, 11, 11)))
    with H.File(p, "cw") as f:
        f["symmetry"] = "u1-dm"
        f["S"] = 0.5
        f["finished"] = True
        f["reduced_lattice/size"] = 3
        f["reduced_lattice/J/1"] = np.array([1.0, 0.8, 0.2])
        f["a/50.0/Γ/Γxx/ch_s/q3"] = q3
        for k in range(700):  # several symbol table nodes and a two-level B-tree
            f[f"χ/{H.julia_float_str(50.0 * 0.99 ** k)}/diag"] = np.full((6, 11), float(k))
    size0 = os.path.getsize(p)
    for k in range(3):
        with H.File(p, "cw") as f:
            f[f"σ/{H.julia_float_str(0.5 + k)}"] = np.arange(5.0) + k
            with pytest.raises(H.HDF5Error):
                f["symmetry"] = "su2"  # existing datasets are never replaced
    assert os.path.getsize(p) - size0 < 64 * 1024  # appends rewrite only the changed groups
    with H.File(p, "r") as f:
        assert f.read("symmetry") == "u1-dm" and f.read("S") == 0.5 and f.read("finished") is True
        assert f.read("reduced_lattice/size") == 3
        assert np.array_equal(f.read("reduced_lattice/J/1"), [1.0, 0.8, 0.2])
        x = f.read("a/50.0/Γ/Γxx/ch_s/q3")
        assert x.shape == q3.shape and np.array_equal(x, q3)
        keys = f.keys("χ")
        assert len(keys) == 700 and keys == sorted(keys, key=lambda s: s.encode())
        k = H.julia_float_str(50.0 * 0.99 ** 321)
        assert np.all(f.read(f"χ/{k}/diag") == 321.0)
        assert f.keys("σ") == ["0.5", "1.5", "2.5"]


@pytest.mark.parametrize("x,s", [(50.0, "50.0"), (0.01, "0.01"), (1e-5, "1.0e-5"), (1e-4, "0.0001"),
                                 (123456.0, "123456.0"), (1234567.0, "1.234567e6"), (2.5e-7, "2.5e-7"),
                                 (0.1 + 0.2, "0.30000000000000004"), (1e6, "1.0e6")])
def test_julia_float_names(pkg, x, s):
    """Group names of the reference are Julia's string(Λ::Float64)."""
    from pffrg_gb300 import hdf5 as H

    assert H.julia_float_str(x) == s


@pytest.mark.parametrize("symmetry", ["su2", "u1-dm"])
def test_checkpoint_and_observables(pkg, tmp_path, symmetry):
    """checkpoint!/read_checkpoint (checkpoint_{su2,u1_dm}.jl), save_self!/save_χ! (Observable/disk.jl),
    save!/read_lattice (Lattice/disk.jl): same paths, shapes and values back."""
    import pffrg_gb300.workloads as wl
    from pffrg_gb300 import disk as D, hdf5 as H

    if symmetry == "su2":
        w = wl.WORKLOADS["square-L3-1l"]
    else:
        w = wl.Workload("t", "kagome", 3, "kagome-xxz-dm", [[1.0, 0.8, 0.2]], 1, 1.0, 10, 5, 4, 0.1, 3,
                        symmetry="u1-dm")
    lat, r, m, a = wl.build_state(w, num_sigma=10, num_omega=5, num_nu=4)
    cp, obs = str(tmp_path / "run_cp"), str(tmp_path / "run_obs")
    chi = [np.random.default_rng(k).normal(size=(r.num_sites, len(m.chi))) for k in range(3)]
    chi = chi[0] if symmetry == "su2" else chi
    with H.File(cp, "cw") as f:
        D.save_lattice(f, r, False)
        D.checkpoint(f, 1.25, 0.05, m, a)
        D.checkpoint(f, 0.75, 0.04, m, a)
    with H.File(obs, "cw") as f:
        D.save_self(f, 1.25, m, a)
        D.save_chi(f, 1.25, symmetry, m, chi)
    with H.File(cp, "r") as f:
        comps = D.COMP_NAMES[symmetry]
        assert f.keys("a/0.75/Γ") == sorted(comps, key=lambda s: s.encode())
        assert f.keys(f"a/0.75/Γ/{comps[0]}/ch_t") == ["q1", "q2_1", "q2_2", "q3"]
        assert f.read(f"a/0.75/Γ/{comps[0]}/ch_t/q3").shape == (r.num_sites, m.num_omega, m.num_nu, m.num_nu)
        lat2, r2 = D.read_lattice(f)
        Lam, dLam, m2, a2 = D.read_checkpoint(f, 0.0)
    assert (Lam, dLam) == (0.75, 0.04) and r2.num_sites == r.num_sites
    assert np.array_equal(a2.buf, a.buf) and np.array_equal(m2.omega_t, m.omega_t)
    with H.File(obs, "r") as f:
        assert D.read_chi_labels(f) == sorted(D.CHI_LABELS[symmetry])
        mesh, mats = D.read_chi_all(f, 1.0, verbose=False)
        assert np.array_equal(mesh, m.chi)
        sig, Sig = D.read_self(f, 1.25)
        assert np.array_equal(Sig, a.Σ)
