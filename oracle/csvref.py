"""rapidcsv's CSV tokenizer, restated -- TEST INFRASTRUCTURE ONLY.

The reference reads both tables with
``rapidcsv::Document(path, LabelParams(-1, -1), SeparatorParams(sep))``
(core/components/data_mngr.h:48-51), so the header line is an ordinary data
row and every cell is read as ``std::string`` (data_mngr.h:61-64).
rapidcsv is a git submodule that the reference does not vendor
(.gitmodules:10-12); its README requires rapidcsv >= 8.65.  This module
restates the published parse of rapidcsv 8.x with the default
SeparatorParams (pTrim=false, pHasCR=false on Linux, pQuotedLinebreaks=false,
pAutoQuote=true) and LineReaderParams (no comment or empty-line skipping):

* a UTF-8 byte-order mark at the start of the file is skipped;
* a double quote toggles the quoted state only when the cell is empty or
  starts with a quote, and is kept in the cell;
* the separator ends a cell unless quoted;
* CR is dropped; LF ends the row (and clears the quoted state);
* a final row without LF is kept;
* each finished cell whose first and last characters are quotes (length >= 2)
  loses them, and doubled quotes inside become single quotes.

Parity of rapidcsv edge cases is pinned only by this restatement; the
synthetic inputs used for parity stay inside the unambiguous subset.
"""
from __future__ import annotations

from typing import List

_BOM = b"\xef\xbb\xbf"


def _unquote(cell: bytes) -> bytes:
    if len(cell) >= 2 and cell[:1] == b'"' and cell[-1:] == b'"':
        return cell[1:-1].replace(b'""', b'"')
    return cell


def parse_rows(data: bytes, sep: bytes = b",") -> List[List[bytes]]:
    """Rows of cells exactly as rapidcsv 8.x stores them (mData)."""
    if data.startswith(_BOM):
        data = data[3:]
    sepc = sep[0]
    rows: List[List[bytes]] = []
    row: List[bytes] = []
    cell = bytearray()
    quoted = False
    for ch in data:
        if ch == 0x22:  # '"'
            if len(cell) == 0 or cell[0] == 0x22:
                quoted = not quoted
            cell.append(ch)
        elif ch == sepc:
            if not quoted:
                row.append(_unquote(bytes(cell)))
                cell.clear()
            else:
                cell.append(ch)
        elif ch == 0x0D:  # '\r' dropped
            pass
        elif ch == 0x0A:
            row.append(_unquote(bytes(cell)))
            rows.append(row)
            cell.clear()
            row = []
            quoted = False
        else:
            cell.append(ch)
    if len(cell) or row:
        row.append(_unquote(bytes(cell)))
        rows.append(row)
    return rows


def read_columns(path: str, sep: str = ",") -> List[List[bytes]]:
    """Column-major cells as DataMngr holds them (data_mngr.h:58-64).

    The column count is the cell count of the first row; a shorter row makes
    rapidcsv's GetColumn throw, so it raises ValueError here.
    """
    with open(path, "rb") as f:
        rows = parse_rows(f.read(), sep.encode()[:1])
    if not rows:
        return []
    n_cols = len(rows[0])
    cols: List[List[bytes]] = [[] for _ in range(n_cols)]
    for ri, r in enumerate(rows):
        if len(r) < n_cols:
            raise ValueError(f"{path}: row {ri} has {len(r)} cells, expected {n_cols}")
        for c in range(n_cols):
            cols[c].append(r[c])
    return cols
