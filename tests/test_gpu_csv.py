"""CSV files of at least 1 MiB read with a context are tokenized on the device
(csv_gpu.cu); every column, byte for byte, equals the host tokenizer's
(csv.cpp, rapidcsv's rules with the reference's parameters): quoted cells
holding the separator, "" escapes, quotes inside unquoted cells, '\\r' bytes
anywhere, empty cells, a UTF-8 BOM, a last row without a line break, rows
with extra cells, other separators; short rows fail the same way."""
import numpy as np
import pytest

import hyperblocker_gb300 as hb

pytestmark = pytest.mark.gpu

ALPHA = b"abcdefghij XYZ0123456789"


def _cell(rng, sep):
    k = int(rng.integers(0, 10))
    body = bytes(rng.choice(list(ALPHA), size=int(rng.integers(0, 30))).tolist())
    if k == 0:
        return b""
    if k == 1:  # quoted, holding the separator and an escaped quote
        return b'"' + body[:5] + sep + b'""' + body[5:] + b'"'
    if k == 2:  # a quote inside an unquoted cell is an ordinary byte
        return b"a" + body[:3] + b'"' + body[3:]
    if k == 3:  # carriage returns are dropped wherever they are
        return body[:2] + b"\r" + body[2:]
    if k == 4:
        return b'"' + body + b'"'
    if k == 5:  # quotes that do not close the cell
        return b'"' + body + b'"x'
    return body


def _csv(rng, n_rows, n_cols, sep, bom=False, tail=True):
    lines = []
    for r in range(n_rows):
        cells = [_cell(rng, sep) for _ in range(n_cols)]
        if r > 0 and rng.random() < 0.02:
            cells.append(b"extra")  # ignored
        line = sep.join(cells)
        if rng.random() < 0.1:
            line += b"\r"
        lines.append(line)
    data = b"\n".join(lines) + (b"\n" if tail else b"")
    return (b"\xef\xbb\xbf" if bom else b"") + data


def _columns(t):
    return [t.column(c) for c in range(t.n_cols)]


@pytest.mark.parametrize("sep,bom,tail", [(b",", False, True), (b",", True, False),
                                          (b";", False, True), (b"\t", True, True)])
def test_device_tokenizer_equals_host(ctx, tmp_path, sep, bom, tail):
    rng = np.random.Generator(np.random.PCG64(len(sep) + 2 * bom + 4 * tail + ord(sep)))
    data = _csv(rng, 40_000, 5, sep, bom, tail)
    assert len(data) >= (1 << 20)
    p = tmp_path / "t.csv"
    p.write_bytes(data)
    host = hb.Table.from_csv(str(p), sep.decode())
    dev = hb.Table.from_csv(str(p), sep.decode(), ctx)
    assert dev.n_rows == host.n_rows and dev.n_cols == host.n_cols
    for (hb_, ho), (db, do) in zip(_columns(host), _columns(dev)):
        assert np.array_equal(ho, do)
        assert np.array_equal(hb_, db)


def test_long_rows_read_from_device_memory(ctx, tmp_path):
    """Groups of 32 rows longer than a warp's 8 KB staging area are walked
    in device memory; they sit between short groups that are staged."""
    rng = np.random.Generator(np.random.PCG64(11))
    rows = _csv(rng, 40_000, 4, b",").split(b"\n")
    for r in list(range(3200, 3264)) + list(range(20_031, 20_040)) + [39_999]:
        long = b'"' + b"x," * int(rng.integers(200, 700)) + b'""y"'
        rows[r] = long + b',"a,b",c\r,' + str(r).encode()
    p = tmp_path / "t.csv"
    p.write_bytes(b"\n".join(rows))
    host = hb.Table.from_csv(str(p))
    dev = hb.Table.from_csv(str(p), ",", ctx)
    assert dev.n_rows == host.n_rows and dev.n_cols == host.n_cols
    for (hb_, ho), (db, do) in zip(_columns(host), _columns(dev)):
        assert np.array_equal(ho, do)
        assert np.array_equal(hb_, db)


def test_runs_of_quotes_separators_and_carriage_returns(ctx, tmp_path):
    """One column of cells drawn from '"', ',', '\\r', 'a', 'b': runs of
    quotes of every length, separators inside and outside quotes, carriage
    returns between a quote and its pair; every row is valid with one
    column (extra cells are ignored)."""
    rng = np.random.Generator(np.random.PCG64(21))
    alpha = np.frombuffer(b'"",\rab', dtype=np.uint8)
    rows = [b"h"]
    for _ in range(90_000):
        rows.append(alpha[rng.integers(0, len(alpha), size=int(rng.integers(0, 28)))].tobytes())
    data = b"\n".join(rows) + b"\n"
    assert len(data) >= (1 << 20)
    p = tmp_path / "t.csv"
    p.write_bytes(data)
    host = hb.Table.from_csv(str(p))
    dev = hb.Table.from_csv(str(p), ",", ctx)
    assert dev.n_rows == host.n_rows and dev.n_cols == host.n_cols == 1
    (hb_, ho), (db, do) = host.column(0), dev.column(0)
    assert np.array_equal(ho, do)
    assert np.array_equal(hb_, db)


def test_tail_of_carriage_returns_is_no_row(ctx, tmp_path):
    rng = np.random.Generator(np.random.PCG64(3))
    data = _csv(rng, 40_000, 3, b",") + b"\r\r"
    p = tmp_path / "t.csv"
    p.write_bytes(data)
    host = hb.Table.from_csv(str(p))
    dev = hb.Table.from_csv(str(p), ",", ctx)
    assert dev.n_rows == host.n_rows == 40_000


def test_short_row_fails_like_the_host(ctx, tmp_path):
    rng = np.random.Generator(np.random.PCG64(4))
    rows = _csv(rng, 40_000, 4, b",").split(b"\n")
    rows[12345] = b"only,two"
    p = tmp_path / "t.csv"
    p.write_bytes(b"\n".join(rows))
    with pytest.raises(hb.HbxError) as eh:
        hb.Table.from_csv(str(p))
    with pytest.raises(hb.HbxError) as ed:
        hb.Table.from_csv(str(p), ",", ctx)
    assert "row 12345 has 2 cells, expected 4" in str(eh.value)
    assert "row 12345 has 2 cells, expected 4" in str(ed.value)
