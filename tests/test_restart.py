"""Restart files (reference SavePsiFile / ReadPsiFile, src/Restart.f90:614-793):
host code, checked here without a GPU against the oracle's restatement of
the gfortran record layout, in both directions, with the reference's
accept/reject rules."""
import os
import struct

import numpy as np
import pytest

import oracle
from mlcp_gb300 import restart as RS


def _block(rng, nev, rk, nbas):
    nD = int(np.sum(nbas))
    return rng.normal(size=(nev, rk, nD)), rng.uniform(0.1, 2.0, size=(nev, rk))


def _state(rng, nev=5, rk=4, nbas=(3, 5, 2, 4)):
    base, coef = _block(rng, nev, rk, nbas)
    return dict(isavi=7, bounds=np.array([-1.5, 42.25]), eigv=np.sort(rng.normal(size=nev)),
                delta=rng.uniform(0, 1e-3, nev), base=base, coef=coef, nbas=np.array(nbas))


def test_save_matches_oracle_reader(tmp_path):
    rng = np.random.default_rng(1)
    s = _state(rng)
    p = tmp_path / "a.rst"
    RS.save_psi_file(p, s["isavi"], s["bounds"], s["eigv"], s["delta"], s["base"], s["coef"], s["nbas"])
    recs = oracle.fortran_records(p)
    assert len(recs) == 4 + 4 * s["eigv"].size
    o = oracle.psi_read(p)
    assert o["isavi"] == 7
    assert np.array_equal(o["bounds"], s["bounds"])
    assert np.array_equal(o["eigv"], s["eigv"]) and np.array_equal(o["delta"], s["delta"])
    assert all(np.array_equal(nb, s["nbas"]) for nb in o["nbas"])
    assert np.array_equal(o["ranks"], [4] * 5)
    assert np.array_equal(o["coef"], s["coef"].ravel())
    assert np.array_equal(o["base"], s["base"].ravel())
    # byte-identical to the oracle's writer
    q = tmp_path / "b.rst"
    oracle.psi_write(q, 7, s["bounds"], s["eigv"], s["delta"], s["nbas"], [4] * 5, s["coef"], s["base"])
    assert p.read_bytes() == q.read_bytes()


def test_read_oracle_file_with_mixed_ranks(tmp_path):
    rng = np.random.default_rng(2)
    nbas = np.array([4, 3, 6])
    nD = int(nbas.sum())
    ranks = [3, 1, 6, 2]
    coef = rng.normal(size=sum(ranks))
    base = rng.normal(size=sum(ranks) * nD)
    p = tmp_path / "m.rst"
    oracle.psi_write(p, 12, [0.5, 9.0], [1.0, 2.0, 3.0, 4.0], [1e-4, 2e-4, 3e-4, 4e-4], nbas, ranks, coef, base)
    st = RS.read_psi_file(p, 4, nbas, max_terms=20)
    assert st is not None and st.isavi == 12
    assert np.array_equal(st.ranks, ranks)
    assert np.array_equal(st.coef, coef) and np.array_equal(st.base, base)
    assert np.array_equal(st.bounds, [0.5, 9.0])
    with pytest.raises(ValueError):
        st.block()
    # capacity below the file's terms reads as a mismatch
    assert RS.read_psi_file(p, 4, nbas, max_terms=11) is None
    assert RS.read_psi_file(p, 4, nbas, max_terms=12) is not None


def test_round_trip_block(tmp_path):
    rng = np.random.default_rng(3)
    s = _state(rng, nev=8, rk=6, nbas=(10, 10, 10))
    p = tmp_path / "r.rst"
    RS.save_psi_file(p, 3, s["bounds"], s["eigv"], s["delta"], s["base"], s["coef"], s["nbas"])
    st = RS.read_psi_file(p, 8, s["nbas"], max_terms=48)
    b, c = st.block()
    assert np.array_equal(b, s["base"]) and np.array_equal(c, s["coef"])


@pytest.mark.parametrize("case", ["nev", "ndof", "nbas", "truncated", "missing", "markers"])
def test_rejects_as_reference(tmp_path, case):
    """Each condition that sets success = .FALSE. in ReadPsiFile leaves the
    caller's data unchanged and reports no success."""
    rng = np.random.default_rng(4)
    s = _state(rng)
    p = tmp_path / "x.rst"
    RS.save_psi_file(p, 1, s["bounds"], s["eigv"], s["delta"], s["base"], s["coef"], s["nbas"])
    nev, nbas = 5, s["nbas"]
    if case == "nev":
        nev = 4
    elif case == "ndof":
        nbas = np.array([3, 5, 6])
    elif case == "nbas":
        nbas = np.array([3, 5, 2, 5])
    elif case == "truncated":
        data = p.read_bytes()
        p.write_bytes(data[:len(data) - 9])
    elif case == "missing":
        p = tmp_path / "absent.rst"
    elif case == "markers":
        data = bytearray(p.read_bytes())
        data[-1] ^= 0x10  # trailing marker of the last record
        p.write_bytes(bytes(data))
    assert RS.read_psi_file(p, nev, nbas, max_terms=40) is None


def test_longer_record_reads_as_fortran(tmp_path):
    """A Fortran READ takes the leading items of a longer record; the first
    record with a trailing extra integer still reads."""
    rng = np.random.default_rng(6)
    s = _state(rng, nev=2, rk=2, nbas=(3, 3))
    p = tmp_path / "l.rst"
    oracle.psi_write(p, 5, s["bounds"], s["eigv"], s["delta"], s["nbas"], [2, 2], s["coef"], s["base"])
    data = p.read_bytes()
    first = struct.pack("<iiii", 12, 5, 2, 99) + struct.pack("<i", 12)
    p.write_bytes(first + data[16:])
    st = RS.read_psi_file(p, 2, s["nbas"], max_terms=4)
    assert st is not None and st.isavi == 5 and np.array_equal(st.coef, s["coef"].ravel())


def test_two_file_scheme(tmp_path, monkeypatch):
    """SavePsi writes _1 and _2; ReadPsi falls back to _2 when _1 is bad, and
    resfile 'none' saves nothing."""
    rng = np.random.default_rng(7)
    s = _state(rng, nev=3, rk=2, nbas=(4, 4))
    res = str(tmp_path / "job")
    RS.save_psi(res, 9, s["bounds"], s["eigv"], s["delta"], s["base"], s["coef"], s["nbas"])
    assert os.path.exists(res + "_1_psi.rst") and os.path.exists(res + "_2_psi.rst")
    with open(res + "_1_psi.rst", "r+b") as f:
        f.truncate(20)
    st = RS.read_psi(res, 3, s["nbas"], max_terms=6)
    assert st is not None and st.isavi == 9 and np.array_equal(st.delta, s["delta"])
    assert RS.read_psi(res, 3, s["nbas"], max_terms=6, dorestart=False) is None
    monkeypatch.chdir(tmp_path)
    RS.save_psi("none", 1, s["bounds"], s["eigv"], s["delta"], s["base"], s["coef"], s["nbas"])
    assert not any(n.startswith("none") for n in os.listdir(tmp_path))
