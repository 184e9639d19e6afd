"""Pair lines formatted on the device (hbx_write_pairs_device, and
hbx_write_pairs with a context and many pairs) are byte-identical to the host
writer's: ids cut at their first NUL, commas and quotes kept, empty ids,
long ids, many chunks, append mode, and out-of-range rows refused."""
import numpy as np
import pytest

import hyperblocker_gb300 as hb

pytestmark = pytest.mark.gpu


def _ids(rng, n, prefix):
    out = [b"id"]
    for i in range(n):
        k = int(rng.integers(0, 6))
        if k == 0:
            out.append(b"")
        elif k == 1:
            out.append(prefix + str(i).encode() + b"\x00tail")  # printed up to the NUL
        elif k == 2:
            out.append(b'"q,' + str(i).encode() + b'"')
        elif k == 3:
            out.append(bytes(rng.integers(33, 127, size=int(rng.integers(40, 120))).astype(np.uint8)))
        else:
            out.append(prefix + str(i).encode())
    return out


def _table(rng, n, prefix, ctx):
    ids = _ids(rng, n, prefix)
    other = [b"x"] + [b"v" for _ in range(n)]
    return hb.Table.from_columns([ids, other], ctx)


def _host_bytes(L, R, pairs, path):
    hb.write_pairs(L, R, pairs, str(path))  # no context: the host loop
    return path.read_bytes()


@pytest.mark.parametrize("n_pairs", [1, 5000, 700_000])
def test_device_lines_equal_host_lines(ctx, tmp_path, n_pairs):
    import torch

    rng = np.random.Generator(np.random.PCG64(77 + n_pairs))
    L = _table(rng, 3000, b"l", ctx)
    R = _table(rng, 5000, b"r", ctx)
    pairs = np.stack([rng.integers(0, 3001, size=n_pairs), rng.integers(0, 5001, size=n_pairs)],
                     axis=1).astype(np.uint32)
    want = _host_bytes(L, R, pairs, tmp_path / "host.txt")
    dl = torch.from_numpy(pairs[:, 0].astype(np.int32)).cuda()
    dr = torch.from_numpy(pairs[:, 1].astype(np.int32)).cuda()
    out = tmp_path / "dev.txt"
    hb.write_pairs_device(ctx, L, R, dl.data_ptr(), dr.data_ptr(), n_pairs, str(out))
    assert out.read_bytes() == want
    # append mode: a second call adds the same lines again
    hb.write_pairs_device(ctx, L, R, dl.data_ptr(), dr.data_ptr(), n_pairs, str(out))
    assert out.read_bytes() == want + want
    # with a context, hbx_write_pairs formats many pairs on the device
    via = tmp_path / "via.txt"
    hb.write_pairs(L, R, pairs, str(via), ctx)
    assert via.read_bytes() == want


def test_many_chunks_of_long_ids(ctx, tmp_path):
    import torch

    rng = np.random.Generator(np.random.PCG64(5))
    n = 2000
    long_ids = [b"id"] + [bytes([65 + i % 26]) * 1000 + str(i).encode() for i in range(n)]
    L = hb.Table.from_columns([long_ids, [b"x"] + [b"v"] * n], ctx)
    R = hb.Table.from_columns([long_ids, [b"x"] + [b"v"] * n], ctx)
    m = 100_000  # about 200 MB of text: several 64 MiB chunks
    pairs = np.stack([rng.integers(0, n + 1, size=m), rng.integers(0, n + 1, size=m)],
                     axis=1).astype(np.uint32)
    want = _host_bytes(L, R, pairs, tmp_path / "host.txt")
    dl = torch.from_numpy(pairs[:, 0].astype(np.int32)).cuda()
    dr = torch.from_numpy(pairs[:, 1].astype(np.int32)).cuda()
    out = tmp_path / "dev.txt"
    hb.write_pairs_device(ctx, L, R, dl.data_ptr(), dr.data_ptr(), m, str(out))
    assert out.read_bytes() == want


def test_out_of_range_rows_are_refused(ctx, tmp_path):
    import torch

    rng = np.random.Generator(np.random.PCG64(9))
    L = _table(rng, 10, b"l", ctx)
    R = _table(rng, 10, b"r", ctx)
    dl = torch.tensor([0, 11], dtype=torch.int32, device="cuda")  # 11 rows with the header
    dr = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    with pytest.raises(hb.HbxError):
        hb.write_pairs_device(ctx, L, R, dl.data_ptr(), dr.data_ptr(), 2, str(tmp_path / "x.txt"))


def test_cli_pipeline_sorts_and_writes_on_device(built, tmp_path):
    """run_hyperblocker_exec keeps the pairs on the device: the file holds the
    engine's pairs sorted by (left row, right row), byte for byte what the
    host writer makes of them, across many sort tiles and row bytes."""
    import subprocess

    from hyperblocker_gb300 import synth
    from tests import _util

    cl, cr = _util.random_tables(3131, 700, 900, b"ab", 12, n_eq_values=2)

    def write_csv(path, cols):
        with open(path, "wb") as f:
            for i in range(len(cols[0])):
                f.write(b",".join(b'"' + c[i] + b'"' for c in cols) + b"\n")

    lp, rp = tmp_path / "l.csv", tmp_path / "r.csv"
    write_csv(lp, cl)
    write_csv(rp, cr)
    rules = tmp_path / "rules"
    rules.mkdir()
    (rules / "0.yaml").write_text(synth.rule_yaml([3], [(1, 0.55)]))
    out = tmp_path / "pairs.csv"
    cmd = [hb.EXE_PATH, "-data_l", str(lp), "-data_r", str(rp), "-rule_dir", str(rules),
           "-n_partitions", "2", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ctx = hb.Context(0)
    plan = hb.Plan.from_rule_dir(str(rules), ctx)
    L = hb.Table.from_csv(str(lp))
    R = hb.Table.from_csv(str(rp))
    pairs, _ = hb.block(ctx, plan, L, R, 2)
    assert len(pairs) > 20_000  # many sort tiles
    want = tmp_path / "want.csv"
    hb.write_pairs(L, R, _util.sorted_pairs(pairs), str(want))  # host loop, row order
    assert out.read_bytes() == want.read_bytes()
    ctx.close()
