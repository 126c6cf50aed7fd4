"""Wave-packet files in the reference's save formats (evr_psi_write / evr_psi_read), on the
host: no GPU needed.

The library's reader and writer are checked against the oracle's restatement of the
Fortran write/read statements (oracle/wpio.py, Source_ElVibRot/sub_WP/sub_module_psi_io.f90)
and against the start packets of the reference's own input files (golden.json "wp_inputs").
Bit-exact: the values pass through text with 17 significant digits, or as raw bytes.
"""
import numpy as np
import pytest

from evrgpu import lib as E
from evrgpu import spec as S
from oracle import oracle as O
from oracle import wpio as W


def _packed(spec):
    return O.OracleProblem(spec).tables()["packed"]


def _block(rng, N, npsi, cplx):
    a = rng.standard_normal((N, npsi))
    if cplx:
        a = a + 1j * rng.standard_normal((N, npsi))
    a[rng.random((N, npsi)) < 0.2] = 0.0  # exact zeros, as a packet on a subset has
    return a


def _two_state_sg4(D=4, L=3):
    p = S.Poly()
    for e in (0, 1):
        for i in range(D):
            p.add(0.5, [i, i], e, e)
    c, idx, el = p.arrays()
    one = np.ones(D, dtype=np.int32)
    return S.ProblemSpec(kind="sg4", D=D, nb0=2, LG=L, LB=L, Aq=one, Bq=2 * one, Ab=one, Bb=2 * one,
                         mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=1)


SPECS = {
    "sg4_hh6d": lambda: S.henon_heiles(6, 3),
    "dp3": lambda: S.config_dp3(nb=6, nq=8),
    "sg4_2state": lambda: _two_state_sg4(),
}


@pytest.mark.parametrize("name", sorted(SPECS))
@pytest.mark.parametrize("fmt", W.FORMATS)
@pytest.mark.parametrize("cplx", [False, True])
def test_round_trip_is_bit_exact(tmp_path, name, fmt, cplx):
    spec = SPECS[name]()
    pg = E.Problem(spec, device=-1)
    psi = _block(np.random.default_rng(3), pg.N, 3, cplx)
    f = tmp_path / f"wp.{fmt}"
    pg.write_psi(f, psi, fmt=fmt)
    back, dropped = pg.read_psi(f, npsi_max=8, cplx=cplx)
    assert dropped == 0 and back.shape == psi.shape
    assert np.array_equal(back, psi)


@pytest.mark.parametrize("fmt", W.FORMATS)
@pytest.mark.parametrize("cplx", [False, True])
def test_library_reads_oracle_files_and_oracle_reads_library_files(tmp_path, fmt, cplx):
    spec = _two_state_sg4(3, 3)
    pg = E.Problem(spec, device=-1)
    packed = _packed(spec)
    psi = _block(np.random.default_rng(11), pg.N, 2, cplx)
    fo = tmp_path / "oracle.wp"
    W.write(fo, fmt, packed, spec.nb0, psi)
    got, dropped = pg.read_psi(fo, npsi_max=4, cplx=cplx)
    assert dropped == 0 and np.array_equal(got, psi)
    fl = tmp_path / "library.wp"
    pg.write_psi(fl, psi, fmt=fmt)
    blk, dropped = W.to_block(W.read(fl, spec.D, cplx), packed, spec.nb0, cplx)
    assert dropped == 0 and np.array_equal(blk, psi)


def test_sparse_form_keeps_entries_at_or_above_epsi(tmp_path):
    spec = S.henon_heiles(6, 3)
    pg = E.Problem(spec, device=-1)
    psi = _block(np.random.default_rng(5), pg.N, 2, True)
    f = tmp_path / "sparse.wp"
    pg.write_psi(f, psi, fmt="sparse", epsi=0.5)
    got, _ = pg.read_psi(f, cplx=True)
    want = np.where(np.abs(psi) >= 0.5, psi, 0.0)
    assert np.array_equal(got, want)
    n_lines = sum(1 for ln in open(f) if ln.strip() and "end" not in ln) - 1
    assert n_lines == int((np.abs(psi) >= 0.5).sum())


def test_reference_input_packets_hcn(golden, tmp_path):
    """Four real start packets of Working_tests/exa_hcn-test/dat_Davidson (no header)."""
    g = golden["wp_inputs"]["hcn_dat_Davidson"]
    spec = S.config_dp3(nb=6, nq=8)
    assert spec.D == g["D"] and spec.nb0 == g["nb0"]
    pg = E.Problem(spec, device=-1)
    packed = _packed(spec)
    f = tmp_path / "dat_packets"
    f.write_text("\n".join(g["lines"]) + "\n")
    got, dropped = pg.read_psi(f, npsi_max=10)
    ref, dref = W.to_block(W.read(f, spec.D, False), packed, spec.nb0, False)
    assert dropped == dref == 0 and got.shape == (pg.N, 4)
    for j, t in enumerate([(1, 1, 1), (2, 1, 1), (1, 2, 1), (1, 1, 2)]):
        r = int(np.flatnonzero((packed == np.array(t)).all(axis=1))[0])
        want = np.zeros(pg.N)
        want[r] = 1.0
        assert np.array_equal(got[:, j], want)
    assert np.array_equal(got, ref)


def test_reference_input_packet_12d_second_state(golden, tmp_path):
    """The complex start packet of MPI_tests/12D_propagation_S0/shell_run, on that test's
    own 12-D pyrazine basis: the ground function of the second electronic state (tuple
    1..1, i_h = 1, i_e = 2), the packet ended by the end of the file."""
    g = golden["wp_inputs"]["pyr12d_shell_run"]
    spec = S.pyrazine_12d(1)
    assert (spec.D, spec.nb0) == (g["D"], g["nb0"])
    pg = E.Problem(spec, device=-1)
    f = tmp_path / "packet"
    f.write_text("\n".join(g["lines"]) + "\n")
    got, dropped = pg.read_psi(f, cplx=True)
    assert dropped == 0 and got.shape == (pg.N, 1)
    want = np.zeros(pg.N, dtype=complex)
    want[pg.Np + 0] = 1.0  # tuple (1,..,1) is packed function 0; state 2 starts at Np
    assert np.array_equal(got[:, 0], want)
    ref, _ = W.to_block(W.read(f, spec.D, True), _packed(spec), spec.nb0, True)
    assert np.array_equal(got, ref)
    # read as real, the line keeps its real part (a list-directed read ignores extra items)
    got_r, _ = pg.read_psi(f, cplx=False)
    assert np.array_equal(got_r[:, 0], want.real)


def test_restart_across_bases(tmp_path):
    """A file of a smaller basis fills the common functions of a larger one; read back on
    the smaller basis, the functions it lacks are dropped and counted."""
    small, large = S.henon_heiles(4, 2), S.henon_heiles(4, 3)
    ps, pl = E.Problem(small, device=-1), E.Problem(large, device=-1)
    ks, kl = _packed(small), _packed(large)
    psi = _block(np.random.default_rng(2), ps.N, 2, False)
    f = tmp_path / "small.wp"
    ps.write_psi(f, psi, fmt="v1")
    got, dropped = pl.read_psi(f)
    assert dropped == 0
    rows = {tuple(t): r for r, t in enumerate(kl)}
    idx = np.array([rows[tuple(t)] for t in ks])
    assert np.array_equal(got[idx], psi)
    rest = np.setdiff1d(np.arange(pl.N), idx)
    assert not got[rest].any()
    big = _block(np.random.default_rng(4), pl.N, 2, False)
    for fmt in W.FORMATS:
        g = tmp_path / f"large.{fmt}"
        pl.write_psi(g, big, fmt=fmt)
        back, dropped = ps.read_psi(g)
        assert dropped == (pl.N - ps.N) * 2, fmt  # epsi = 0 writes every entry, zeros included
        assert np.array_equal(back, big[idx]), fmt


def test_npsi_max_limits_the_packets_read(tmp_path):
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    psi = _block(np.random.default_rng(8), pg.N, 5, False)
    for fmt in W.FORMATS:
        f = tmp_path / f"wp.{fmt}"
        pg.write_psi(f, psi, fmt=fmt)
        got, _ = pg.read_psi(f, npsi_max=2)
        assert np.array_equal(got, psi[:, :2]), fmt


def test_malformed_files_are_rejected(tmp_path):
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    psi = _block(np.random.default_rng(9), pg.N, 2, False)
    cases = {}
    f = tmp_path / "v0"
    pg.write_psi(f, psi, fmt="v0")
    lines = f.read_text().splitlines()
    cases["v0 truncated"] = "\n".join(lines[:-5]) + "\n"
    cases["v0 no end line"] = "\n".join([ln for ln in lines if "end" not in ln]) + "\n"
    g = tmp_path / "v1"
    pg.write_psi(g, psi, fmt="v1")
    v1 = g.read_text()
    cases["v1 open namelist"] = v1.replace(" /\n", "\n", 1)
    cases["v1 version 2"] = v1.replace("VERSION_FILE=1", "VERSION_FILE=2")
    cases["v1 bad value"] = v1[: v1.rfind("E")] + "Zq\n"
    cases["v1 truncated"] = "\n".join(v1.splitlines()[:-2]) + "\n"
    cases["empty"] = ""
    for what, text in cases.items():
        h = tmp_path / "bad"
        h.write_text(text)
        with pytest.raises(E.EvrError) as ei:
            pg.read_psi(h)
        assert ei.value.code == E.EVR_EINVAL, what
    u = tmp_path / "unf"
    pg.write_psi(u, psi, fmt="unformatted")
    b = u.read_bytes()
    u.write_bytes(b[:-3])
    with pytest.raises(E.EvrError):
        pg.read_psi(u)
    u.write_bytes(b)
    with pytest.raises(E.EvrError) as ei:  # real packets read as complex: record size differs
        pg.read_psi(u, cplx=True)
    assert ei.value.code == E.EVR_EINVAL
    with pytest.raises(E.EvrError):
        pg.read_psi(tmp_path / "missing")
    with pytest.raises(E.EvrError):
        pg.write_psi(tmp_path / "x", psi[:-1], fmt="v0")


def test_unformatted_file_with_8_byte_integers(tmp_path):
    """A build with 8-byte default integers (the reference's long-integer tests) writes the
    header and index records with 8-byte integers; the reader takes their width from the
    nb_psi record."""
    import struct
    spec = S.henon_heiles(3, 2)
    pg = E.Problem(spec, device=-1)
    packed = _packed(spec)
    psi = _block(np.random.default_rng(6), pg.N, 2, False)

    def rec(b):
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))

    out = [rec(b"X"), rec(struct.pack("<q", 2)), rec(struct.pack("<q", pg.N)), rec(struct.pack("<q", 1)), rec(b"X")]
    out += [rec(struct.pack(f"<{spec.D + 2}q", *t)) for t in W.tuples(packed, spec.nb0)]
    out += [rec(np.ascontiguousarray(psi[:, j]).tobytes()) for j in range(2)]
    f = tmp_path / "long_int.wp"
    f.write_bytes(b"".join(out))
    got, dropped = pg.read_psi(f)
    assert dropped == 0 and np.array_equal(got, psi)


def test_restart_file_round_trip_and_oracle(tmp_path):
    """SaveWP_restart / ReadWP_restart: bit-exact round trip, files of the restated Fortran
    statements read by the library and the library's read by them."""
    pg = E.Problem(_two_state_sg4(3, 3), device=-1)
    psi = _block(np.random.default_rng(12), pg.N, 3, True)
    f = tmp_path / "restart"
    pg.write_restart(f, 1234.5678901234567, psi)
    t, back = pg.read_restart(f, 3)
    assert t == 1234.5678901234567 and np.array_equal(back, psi)
    t2, b2 = W.read_restart(f, 3)
    assert t2 == t and np.array_equal(b2, psi)
    g = tmp_path / "restart_oracle"
    W.write_restart(g, 10.0, psi)
    t3, b3 = pg.read_restart(g, 3)
    assert t3 == 10.0 and np.array_equal(b3, psi)


def test_restart_file_absent_header_and_size_mismatch(tmp_path):
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    f = tmp_path / "empty_restart"
    f.write_text("\n")
    assert pg.read_restart(f, 1) == (0.0, None)  # no restart: start at T = 0
    psi = _block(np.random.default_rng(13), pg.N, 2, True)
    g = tmp_path / "restart"
    pg.write_restart(g, 5.0, psi)
    with pytest.raises(E.EvrError) as ei:  # two packets in the file, one requested
        pg.read_restart(g, 1)
    assert ei.value.code == E.EVR_EINVAL
    g.write_text("\n".join(g.read_text().splitlines()[:-3]) + "\n")
    with pytest.raises(E.EvrError):
        pg.read_restart(g, 2)


def test_autocorr_file(tmp_path):
    rng = np.random.default_rng(14)
    t = np.arange(7) * 4.134
    c = rng.standard_normal(7) + 1j * rng.standard_normal(7)
    f = tmp_path / "file_auto"
    E.write_autocorr(f, t[:4], c[:4])
    E.write_autocorr(f, t[4:], c[4:], append=True)
    with open(f, "a") as h:
        h.write(" not an autocorrelation line\n")
    tt, cc = E.read_autocorr(f)
    assert np.array_equal(tt, t) and np.array_equal(cc, c)
    to, co = W.read_autocorr(f)
    assert np.array_equal(to, t) and np.array_equal(co, c)
    g = tmp_path / "file_auto_oracle"
    W.write_autocorr(g, t, c)
    tt, cc = E.read_autocorr(g)
    assert np.array_equal(tt, t) and np.array_equal(cc, c)


def test_fortran_list_directed_variants(tmp_path):
    """Forms other compilers write: the namelist on one line with spaces around '=', D
    exponents, repeat counts r*x, an exponent without its letter (1.5-100), comma
    separators and CRLF line ends."""
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    packed = _packed(S.henon_heiles(3, 2))
    N = pg.N
    want = np.zeros(N)
    want[0], want[1], want[2], want[3] = 0.5, -2.0, 1.5e-100, 3.0
    vals = ["5.0D-01", "-2.0d0", "1.5-100", "3.0E+000"] + ([f"{N - 4}*0.0"] if N > 4 else [])
    lines = [" &headerFile Version_File = 1, nb_psi = 1, nb_tot = %d /" % N]
    lines += [" ".join(str(x) for x in t) for t in W.tuples(packed, 1)]
    lines += [", ".join(vals)]
    f = tmp_path / "variants.wp"
    f.write_bytes(("\r\n".join(lines) + "\r\n").encode())
    got, dropped = pg.read_psi(f)
    assert dropped == 0 and got.shape == (N, 1)
    assert np.array_equal(got[:, 0], want)
    # complex values with a repeat count and blanks inside the parentheses
    lines[-1] = "( 1.0D0 , -2.0 ) %d*(0.0,0.0)" % (N - 1)
    f.write_text("\n".join(lines) + "\n")
    got, _ = pg.read_psi(f, cplx=True)
    assert got[0, 0] == 1.0 - 2.0j and not got[1:, 0].any()
