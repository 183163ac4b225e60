"""Shared-memory layout of the FP32 predictor's flux buffer (PredCfg in
ader-dg_gb300/csrc/predictor.cuh), restated here and checked on the CPU.

A 16-byte shared-memory access of a warp is served in four phases of eight
lanes; a phase costs one wavefront per distinct address in its busiest
16-byte bank group (eight groups of four banks), so the eight lanes of a phase
cost one wavefront when their addresses fall in eight different groups or
coincide. The tests check, for every Euler / Baer-Nunziato degree:
- the row/column pass (P >= 4) and the node accesses around it (flux stores,
  read-back) take one wavefront per phase, and the contractions of the first
  and last Picard iterations take one at P <= 4;
- every (time level, row) and (time level, column) pair is contracted by
  exactly one thread of a cell;
- every address stays inside its cell's slot, and the buffer leaves room for
  the epilogue's [V][P2] x 3 layout.
"""
import pytest

EULER, BN = 1, 2


def pred_cfg(system, N):
    """FP32 PredCfg constants (float4 units unless noted)."""
    P = N + 1
    P2 = P * P
    V = 4 if system == EULER else 9
    VF = 8 if (system == BN and N <= 4) else V
    VP = (VF + 3) // 4 * 4
    NCH = VP // 4
    rowcol = P >= 4
    XL = P2 + (0 if P == 5 else 1) if rowcol else 2 * P2
    YL = P2 + (4 if P == 5 else 2) if rowcol else 2 * P2
    Y0 = P * XL if rowcol else P2
    PC = (1 if P == 2 else 0) if (not rowcol and system == BN) else 0
    if rowcol:
        CE = (5 if system == BN else 3) if P == 5 else (2 if (P == 6 and system == EULER) else 0)
    elif system == BN:
        CE = 1 if P == 3 else 0
    else:
        CE = {2: 4, 3: 6}.get(P, 0)
    PLANE = (Y0 + P * YL if rowcol else 2 * P * P2) + PC
    flux = 4 * NCH * PLANE                     # floats
    raw = flux + (P * P2 if system == BN else 0)
    cell = (raw + 3) // 4 * 4 + 4 * CE         # floats
    cpb = max(1, min((128 if N <= 4 else 256) // P2, (100 * 1024) // (cell * 4)))
    threads = (cpb * P2 + 31) // 32 * 32
    return dict(P=P, P2=P2, V=V, NCH=NCH, rowcol=rowcol, XL=XL, YL=YL, Y0=Y0, PLANE=PLANE, CELL4=cell // 4,
                cell=cell, flux=flux, cpb=cpb, threads=threads)


def layout(c):
    """float4 offset, within a cell, of chunk ch of the flux of direction d,
    time level l, node (x, y)."""
    def a(ch, d, l, x, y):
        off = l * c["XL"] if d == 0 else c["Y0"] + l * c["YL"]
        return c["PLANE"] * ch + off + x + c["P"] * y
    return a


def lanes(c):
    """(slot, i, j) of every thread, warp by warp; the tail threads share the scratch slot."""
    P2, P = c["P2"], c["P"]
    out = []
    for t in range(c["threads"]):
        lc = min(t // P2, c["cpb"])
        node = t - (t // P2) * P2
        out.append((lc, node % P, node // P))
    return [out[w:w + 32] for w in range(0, len(out), 32)]


def wavefronts(addrs):
    tot = 0
    for ph in range(4):
        a = set(addrs[ph * 8: ph * 8 + 8])
        groups = {}
        for x in a:
            groups.setdefault(x % 8, set()).add(x)
        tot += max(len(g) for g in groups.values())
    return tot / 4


CASES = [(s, N) for s in (EULER, BN) for N in (1, 2, 3, 4, 5)]


@pytest.mark.parametrize("system,N", CASES)
def test_flux_buffer_bank_groups(system, N):
    c = pred_cfg(system, N)
    a = layout(c)
    P = c["P"]
    worst = {}

    def acc(name, addrs):
        worst[name] = max(worst.get(name, 0), wavefronts(addrs))

    for warp in lanes(c):
        base = [lc * c["CELL4"] for lc, _, _ in warp]
        for ch in range(c["NCH"]):
            for l in range(P):
                for d in (0, 1):
                    acc("node", [b + a(ch, d, l, i, j) for b, (_, i, j) in zip(base, warp)])
            for k in range(P):
                acc("x", [b + a(ch, 0, 0, k, j) for b, (_, i, j) in zip(base, warp)])
                acc("y", [b + a(ch, 1, 0, i, k) for b, (_, i, j) in zip(base, warp)])
                if c["rowcol"]:
                    acc("row", [b + a(ch, 0, i, k, j) for b, (_, i, j) in zip(base, warp)])
                    if P >= 5:
                        acc("col", [b + a(ch, 1, j, i, k) for b, (_, i, j) in zip(base, warp)])
                    else:
                        acc("col", [b + a(ch, 1, i, j, k) for b, (_, i, j) in zip(base, warp)])
    if c["rowcol"]:
        assert worst["node"] == 1 and worst["row"] == 1 and worst["col"] == 1, worst
    if P <= 4:
        assert worst["x"] == 1 and worst["y"] == 1, worst


@pytest.mark.parametrize("system,N", [(s, N) for s, N in CASES if N >= 3])
def test_row_column_pass_covers_each_line_once(system, N):
    c = pred_cfg(system, N)
    P = c["P"]
    rows, cols = set(), set()
    for i in range(P):
        for j in range(P):
            rows.add((i, j))                                     # level i, row j
            cols.add((j, i) if P >= 5 else (i, j))               # (level, column)
    assert len(rows) == P * P and len(cols) == P * P
    a = layout(c)
    touched = set()
    for ch in range(c["NCH"]):
        for lv, r in rows:
            for k in range(P):
                x = a(ch, 0, lv, k, r)
                assert x < c["PLANE"] * ch + c["Y0"]             # x rows stay in the x levels
                touched.add(x)
        for lv, col in cols:
            for k in range(P):
                y = a(ch, 1, lv, col, k)
                assert c["PLANE"] * ch + c["Y0"] <= y < c["PLANE"] * (ch + 1)
                touched.add(y)
    # every node of every level and direction is contracted exactly once
    assert len(touched) == c["NCH"] * 2 * P * P * P


@pytest.mark.parametrize("system,N", CASES)
def test_flux_buffer_fits_the_cell_slot(system, N):
    c = pred_cfg(system, N)
    a = layout(c)
    P = c["P"]
    top = max(a(ch, d, l, x, y) for ch in range(c["NCH"]) for d in (0, 1) for l in range(P)
              for x in range(P) for y in range(P))
    assert 4 * (top + 1) <= c["flux"] <= c["cell"]
    assert c["cell"] >= 3 * c["V"] * c["P2"]                   # epilogue Q, FX, FY [V][P2]
    assert c["cell"] % 4 == 0 and c["cpb"] * c["cell"] * 4 <= 100 * 1024 or c["cpb"] == 1


def mma_lines(c):
    """(base, stride) in floats of every line of mma_pass (predictor.cuh): line
    L (component v fastest) = (cell, chunk, direction, level, row or column, v)."""
    P, out = c["P"], []
    for L in range(c["cpb"] * c["NCH"] * 2 * P * P * 4):
        v, r1 = L & 3, L >> 2
        r, r2 = r1 % P, r1 // P
        lv, r3 = r2 % P, r2 // P
        d, r4 = r3 & 1, r3 >> 1
        ch, cell = r4 % c["NCH"], r4 // c["NCH"]
        cb = cell * c["cell"] + ch * 4 * c["PLANE"] + v
        if d == 0:
            out.append((cb + (lv * c["XL"] + P * r) * 4, 4))
        else:
            out.append((cb + (c["Y0"] + lv * c["YL"] + r) * 4, 4 * P))
    return out


@pytest.mark.parametrize("system,N", [(s, N) for s, N in CASES if N >= 3])
def test_mma_pass_lines_are_the_row_column_lines(system, N):
    """The tensor-core pass contracts the lines of the row/column pass: the
    same elements, each in exactly one line (so that the warps' in-place
    writes never meet), inside the CTA's cell slots."""
    c = pred_cfg(system, N)
    P = c["P"]
    a = layout(c)
    expect = set()
    for cell in range(c["cpb"]):
        for ch in range(c["NCH"]):
            for d in (0, 1):
                for lv in range(P):
                    for x in range(P):
                        for y in range(P):
                            for v in range(4):
                                expect.add(cell * c["cell"] + 4 * a(ch, d, lv, x, y) + v)
    seen = []
    for base, stride in mma_lines(c):
        seen += [base + k * stride for k in range(P)]
    assert len(seen) == len(set(seen)) == len(expect)
    assert set(seen) == expect
    assert max(seen) < c["cpb"] * c["cell"]
    # the A-fragment loads of one tile (row g = lane / 4 reads element lane % 4):
    # shared-memory wavefronts per 32-bit warp access, for the record
    lines = mma_lines(c)
    worst = 0
    for t0 in range(0, len(lines) - 15, 16):
        for half in (0, 8):
            words = [lines[t0 + half + (ln >> 2)][0] + (ln & 3) * lines[t0 + half + (ln >> 2)][1] for ln in range(32)]
            banks = {}
            for w in set(words):
                banks.setdefault(w % 32, set()).add(w)
            worst = max(worst, max(len(b) for b in banks.values()))
    print("system %d N %d: mma_pass A loads, worst %d wavefronts per access" % (system, N, worst))
