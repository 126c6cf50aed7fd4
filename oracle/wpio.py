"""Restatement of the reference's wave-packet file forms, for checking the library's
readers and writers (evr_psi_read / evr_psi_write, evr_restart_*, evr_autocorr_*).

TEST INFRASTRUCTURE ONLY: imported by tests/.  The product library never imports it.

It writes packets as the reference's Fortran statements do under gfortran's
list-directed output (integers in 12-character fields, reals in G form with 17
significant digits and three-digit exponents, complex as (re,im), namelists as
NAME=value lines), and reads the same forms back:
  sub_save_psi + Write_header_saveFile_psi + Write_Psi_nDBasis
      Source_ElVibRot/sub_WP/sub_module_psi_io.f90:365-424, 1441-1498, 1607-1778
  ecri_psiBasisRepnotall_nD   :783-917      (sparse packets, "end wp k" lines)
  Read_header_saveFile_psi    :1294-1439    (the three formatted headers, unformatted)
  SaveWP_restart / ReadWP_restart, Write_AutoCorr / Read_AutoCorr
      Source_ElVibRot/sub_propagation/sub_module_propagation.f90:376-488, 548-578
A function is its tuple n_1..n_D i_h i_e (Rec_ndim_index, sub_module_basis.f90:3156),
taken here from the oracle's packed table, with i_h = 1 and i_e the electronic state.

Pins: the sparse packet form is pinned by the packets of the reference's own input files
(tests/golden/golden.json "wp_inputs").  No file saved by the reference exists in its
tree, so the saved-file forms are restated from the write statements cited above.
"""
from __future__ import annotations

import math
import struct

import numpy as np

FORMATS = ("v0", "v1", "unformatted", "sparse")


def _fi(n: int) -> str:
    return f"{n:12d}"


def _fr(v: float) -> str:
    """One real(8) as gfortran's list-directed output writes it (G form, 17 digits)."""
    v = float(v)
    if v == 0.0:
        return "   0.0000000000000000     "
    e = int(math.floor(math.log10(abs(float(f"{v:.16E}")))))
    if -1 <= e < 17:
        body = f"{v:.{16 - e}f}"
        return " " + body.rjust(24) + "     "
    m, ex = f"{v:.16E}".split("E")
    return " " + f"{m}E{int(ex):+04d}".rjust(24)


def _fc(re: float, im: float) -> str:
    return " (" + _fr(re) + "," + _fr(im) + ")"


def tuples(packed: np.ndarray, nb0: int):
    """(n_1..n_D, i_h, i_e) of every row of a vector, in the reference's i_e, i_h, i_b order."""
    Np, _ = packed.shape
    out = []
    for ie in range(nb0):
        for k in range(Np):
            out.append(tuple(int(x) for x in packed[k]) + (1, ie + 1))
    return out


def write(path, fmt, packed, nb0, psi, epsi=0.0):
    """psi: N x npsi array (real or complex), rows in packed order."""
    psi = np.asarray(psi)
    cplx = np.iscomplexobj(psi)
    N, npsi = psi.shape
    tup = tuples(packed, nb0)
    assert len(tup) == N
    if fmt == "unformatted":
        def rec(b):
            return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))
        out = [rec(b"X"), rec(struct.pack("<i", npsi)), rec(struct.pack("<i", N)), rec(struct.pack("<i", 1)), rec(b"X")]
        for t in tup:
            out.append(rec(struct.pack(f"<{len(t)}i", *t)))
        for j in range(npsi):
            col = np.ascontiguousarray(psi[:, j], dtype=np.complex128 if cplx else np.float64)
            out.append(rec(col.tobytes()))
        with open(path, "wb") as f:
            f.write(b"".join(out))
        return
    lines = []
    if fmt == "v1":
        lines += ["&HEADERFILE", f" VERSION_FILE={1:<10d},", f" NB_PSI={npsi:<10d},", f" NB_TOT={N:<10d},", " /"]
        lines += ["".join(_fi(x) for x in t) for t in tup]
        for j in range(npsi):
            items = [_fc(z.real, z.imag) for z in psi[:, j]] if cplx else [_fr(x) for x in psi[:, j]]
            per = 1 if cplx else 3
            lines += ["".join(items[i:i + per]) for i in range(0, N, per)]
    else:
        lines.append(_fi(npsi) + (_fi(N) if fmt == "v0" else ""))
        for j in range(npsi):
            for r, t in enumerate(tup):
                z = psi[r, j]
                mod = abs(z)
                if fmt == "sparse" and not mod >= epsi:
                    continue
                vals = _fr(z.real) + _fr(z.imag) if cplx else _fr(z)
                lines.append("".join(_fi(x) for x in t) + vals)
            lines.append(" end wp " + _fi(j + 1))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _num(s: str) -> float:
    return float(s.replace("D", "E").replace("d", "E"))


def read(path, D, cplx):
    """Packets of a file as a list of dicts {tuple: value}, in file order."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:5] == b"\x01\x00\x00\x00X":
        recs, pos = [], 0
        while pos < len(raw):
            (m,) = struct.unpack_from("<i", raw, pos)
            recs.append(raw[pos + 4: pos + 4 + m])
            pos += 8 + m
        npsi = struct.unpack("<i", recs[1])[0]
        ntot = struct.unpack("<i", recs[2])[0]
        tup = [struct.unpack(f"<{D + 2}i", recs[5 + e]) for e in range(ntot)]
        dt = np.complex128 if cplx else np.float64
        return [dict(zip(tup, np.frombuffer(recs[5 + ntot + j], dtype=dt))) for j in range(npsi)]
    lines = [ln for ln in raw.decode().splitlines() if ln.strip()]
    if lines[0].strip().startswith("&"):
        hdr, i = {}, 0
        while "/" not in lines[i]:
            for part in lines[i].replace(",", " ").split():
                if "=" in part:
                    k, v = part.split("=")
                    hdr[k.upper()] = int(v)
            i += 1
        i += 1
        npsi, ntot = hdr["NB_PSI"], hdr["NB_TOT"]
        tup = [tuple(int(x) for x in lines[i + e].split()[: D + 2]) for e in range(ntot)]
        i += ntot
        vals = []
        for ln in lines[i:]:
            if cplx:
                for item in ln.replace(" ", "").split(")("):
                    a, b = item.strip("()").split(",")
                    vals.append(complex(_num(a), _num(b)))
            else:
                vals += [_num(x) for x in ln.split()]
        return [dict(zip(tup, vals[j * ntot:(j + 1) * ntot])) for j in range(npsi)]
    head = lines[0].split()
    body = lines[1:] if len(head) <= 2 else lines
    packets, cur = [], {}
    for ln in body:
        p = ln.split()
        if ln.strip().startswith("end"):
            packets.append(cur)
            cur = {}
            continue
        t = tuple(int(x) for x in p[: D + 2])
        cur[t] = complex(_num(p[D + 2]), _num(p[D + 3])) if cplx else _num(p[D + 2])
    if cur:
        packets.append(cur)
    return packets


def to_block(packets, packed, nb0, cplx):
    """Packets ({tuple: value}) as an N x npsi array on the basis of `packed`; entries of
    tuples outside it are dropped and counted."""
    tup = tuples(packed, nb0)
    row = {t: r for r, t in enumerate(tup)}
    out = np.zeros((len(tup), len(packets)), dtype=np.complex128 if cplx else np.float64)
    dropped = 0
    for j, pk in enumerate(packets):
        for t, v in pk.items():
            r = row.get(tuple(t))
            if r is None:
                dropped += 1
            else:
                out[r, j] = v
    return out, dropped


def write_restart(path, t, psi):
    """SaveWP_restart (Source_ElVibRot/sub_propagation/sub_module_propagation.f90:376-424):
    `write(no,*) T,size(WP),size(CvecB)` then `write(no,*) WP(i)%CvecB` per packet."""
    psi = np.asarray(psi, dtype=np.complex128)
    N, npsi = psi.shape
    lines = [_fr(t) + _fi(npsi) + _fi(N)]
    for j in range(npsi):
        lines += [_fc(z.real, z.imag) for z in psi[:, j]]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_restart(path, npsi):
    with open(path) as f:
        lines = f.read().splitlines()
    h = lines[0].split()
    t, nw, n = _num(h[0]), int(h[1]), int(h[2])
    assert nw == npsi
    vals = []
    for ln in lines[1:]:
        for item in ln.replace(" ", "").split(")("):
            if item.strip("()"):
                a, b = item.strip("()").split(",")
                vals.append(complex(_num(a), _num(b)))
    return t, np.array(vals).reshape(npsi, n).T


def write_autocorr(path, t, cdot):
    """Write_AutoCorr (:548-557): `write(no,*) 'AutoCor ',T,real(cdot),aimag(cdot),abs(cdot)`."""
    with open(path, "w") as f:
        for tt, z in zip(t, cdot):
            f.write(" AutoCor " + _fr(tt) + _fr(z.real) + _fr(z.imag) + _fr(abs(z)) + "\n")


def read_autocorr(path):
    t, c = [], []
    with open(path) as f:
        for ln in f:
            p = ln.split()
            if len(p) >= 5 and p[0] == "AutoCor":
                t.append(_num(p[1]))
                c.append(complex(_num(p[2]), _num(p[3])))
    return np.array(t), np.array(c)
