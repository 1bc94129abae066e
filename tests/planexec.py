"""numpy executor for exported tile plans (llg_plan_export): runs each pass over all tiles at
once, so the CPU tests can check the planner's output against the oracle without a GPU."""
from __future__ import annotations

import numpy as np


def _matrix(x) -> np.ndarray:
    k, c = int(x["kind"]), x["c"]
    if k == 0:
        return np.array([[c[0] + 1j * c[1], c[2] + 1j * c[3]], [c[4] + 1j * c[5], c[6] + 1j * c[7]]])
    if k == 1:
        return np.array([[c[0], -1j * c[1]], [-1j * c[1], c[0]]])
    if k == 2:
        return np.array([[c[0], -c[1]], [c[1], c[0]]], dtype=complex)
    if k == 3:
        return np.array([[c[0], c[0]], [c[0], -c[0]]], dtype=complex)
    if k == 12:  # [c, -s; s, c] diag(1, eg)
        eg = c[0] + 1j * c[1]
        return np.array([[c[2], -c[3]], [c[3], c[2]]], dtype=complex) @ np.diag([1, eg])
    if k == 14:  # [1, -t; t, 1] diag(1, eg)
        eg, t = c[0] + 1j * c[1], c[2]
        return np.array([[1, -t], [t, 1]], dtype=complex) @ np.diag([1, eg])
    if k == 15:  # [u, -1; 1, u] diag(1, eg)
        eg, u = c[0] + 1j * c[1], c[2]
        return np.array([[u, -1], [1, u]], dtype=complex) @ np.diag([1, eg])
    if k == 16:  # [1, -t; t, 1] (input phase applied by a phase table)
        return np.array([[1, -c[2]], [c[2], 1]], dtype=complex)
    if k == 17:  # [u, -1; 1, u]
        return np.array([[c[2], -1], [1, c[2]]], dtype=complex)
    if k == 22:  # [1, -it; -it, 1]
        return np.array([[1, -1j * c[2]], [-1j * c[2], 1]])
    if k == 23:  # [u, -i; -i, u]
        return np.array([[c[2], -1j], [-1j, c[2]]])
    if k in (25, 26):  # diag(1, ea) [1, -t; t, 1] diag(1, eg) / diag(1, ea) [u, -1; 1, u] diag(1, eg)
        eg, ea, a = c[0] + 1j * c[1], c[4] + 1j * c[5], c[2]
        r = np.array([[1, -a], [a, 1]] if k == 25 else [[a, -1], [1, a]], dtype=complex)
        return np.diag([1, ea]) @ r @ np.diag([1, eg])
    if k == 24:  # [1, 1; 1, -1]
        return np.array([[1, 1], [1, -1]], dtype=complex)
    if k == 11:  # diag(1, ea) [c, -s; s, c] diag(1, eg)
        eg, ea = c[0] + 1j * c[1], c[4] + 1j * c[5]
        ry = np.array([[c[2], -c[3]], [c[3], c[2]]], dtype=complex)
        return np.diag([1, ea]) @ ry @ np.diag([1, eg])
    return np.array([[0, 1], [1, 0]], dtype=complex)


def _pair(tile: np.ndarray, q: int, m: np.ndarray) -> None:
    nt, size = tile.shape
    v = tile.reshape(nt, size >> (q + 1), 2, 1 << q)
    a0, a1 = v[:, :, 0, :].copy(), v[:, :, 1, :].copy()
    v[:, :, 0, :] = m[0, 0] * a0 + m[0, 1] * a1
    v[:, :, 1, :] = m[1, 0] * a0 + m[1, 1] * a1


def unregister(passes: np.ndarray, xops: np.ndarray) -> np.ndarray:
    """A register program (kind 19 layout ops, register slots in the op records) turned back into
    the tile program it encodes: slots replaced by the layout's local positions, layout ops kept
    as no-ops (kind -1).  Also checks the layouts: four distinct register positions, and thread
    positions covering the rest of the tile."""
    out = xops.copy()
    for p in passes:
        t = int(p["t"])
        regs = list(range(t - 4, t))
        for i in range(int(p["op_begin"]), int(p["op_begin"]) + int(p["nops"])):
            x = out[i]
            k = int(x["kind"])
            if k == 19:
                regs = [(int(x["mask"]) >> (4 * j)) & 15 for j in range(4)]
                thr = [(int(x["nl_mask"]) >> (4 * j)) & 15 for j in range(int(x["q0"]))]
                assert int(x["q0"]) == t - 4 and sorted(regs + thr) == list(range(t)), (regs, thr)
                out[i]["kind"] = -1
            elif k == 6:
                out[i]["q1"] = regs[int(x["q1"])]
                if int(x["flags"]) & 16:
                    out[i]["q0"] = regs[int(x["q0"])]
            elif k in (5, 13):
                if int(x["flags"]) & 16:
                    out[i]["q0"] = regs[int(x["q0"])]
            elif k != 7:
                assert 0 <= int(x["q0"]) < 4
                out[i]["q0"] = regs[int(x["q0"])]
        assert regs == list(range(t - 4, t))  # every pass ends in the base layout
    return out


def execute(psi: np.ndarray, n: int, passes: np.ndarray, xops: np.ndarray, tables: np.ndarray | None = None) -> np.ndarray:
    psi = psi.copy()
    for p in passes:
        lm = int(p["local_mask"])
        t = int(p["t"])
        local = [q for q in range(n) if lm >> q & 1]
        assert len(local) == t
        nonlocal_q = [q for q in range(n) if not lm >> q & 1]
        bases = np.zeros(1 << (n - t), dtype=np.int64)
        for j, q in enumerate(nonlocal_q):
            bases |= ((np.arange(1 << (n - t)) >> j) & 1) << q
        offs = np.zeros(1 << t, dtype=np.int64)
        for j, q in enumerate(local):
            offs |= ((np.arange(1 << t) >> j) & 1) << q
        idx = bases[:, None] | offs[None, :]
        tile = psi[idx]
        lidx = np.arange(1 << t)
        for x in xops[p["op_begin"]:p["op_begin"] + p["nops"]]:
            k, q0, q1, fl = int(x["kind"]), int(x["q0"]), int(x["q1"]), int(x["flags"])
            if k == -1:
                continue
            if k <= 4 or k in (11, 12, 14, 15, 16, 17, 22, 23, 24, 25, 26):
                _pair(tile, q0, _matrix(x))
            elif k == 20:  # 4x4 block on (q0, q1): 16 table entries from `mask`, row-major
                off = int(x["mask"])
                mm = tables[off:off + 16].reshape(4, 4)
                v = tile.reshape(tile.shape[0], -1)
                b0 = ((lidx >> q0) & 1) + 2 * ((lidx >> q1) & 1)
                base_idx = lidx[b0 == 0]
                cols = [base_idx, base_idx | (1 << q0), base_idx | (1 << q1), base_idx | (1 << q0) | (1 << q1)]
                vals = [v[:, c].copy() for c in cols]
                for r in range(4):
                    v[:, cols[r]] = sum(mm[r, k2] * vals[k2] for k2 in range(4))
            elif k == 21:  # 2x2 on q1 chosen by the tile's global control bit q0
                off = int(x["mask"])
                sel = ((bases >> q0) & 1).astype(bool)
                for s_, val in ((~sel, 0), (sel, 1)):
                    sub = tile[s_]
                    _pair(sub, q1, tables[off + 4 * val:off + 4 * val + 4].reshape(2, 2))
                    tile[s_] = sub
            elif k == 18:  # phase table: tile amplitude l times entry l
                off = int(x["mask"])
                tile *= tables[off:off + (1 << t)][None, :]
            elif k == 13:  # diag(1, ph) on q0 (tile-uniform when q0 is not local)
                ph = x["c"][0] + 1j * x["c"][1]
                if fl & 1:
                    sel = ((bases >> q0) & 1).astype(bool)
                    tile[sel] *= ph
                else:
                    bit = ((lidx >> q0) & 1).astype(bool)
                    tile[:, bit] *= ph
            elif k == 5:
                c = x["c"]
                d0, d1 = c[0] + 1j * c[1], c[2] + 1j * c[3]
                if fl & 1:
                    sel = ((bases >> q0) & 1).astype(bool)
                    tile[sel] *= d1
                    tile[~sel] *= d0
                else:
                    bit = ((lidx >> q0) & 1).astype(bool)
                    tile[:, bit] *= d1
                    tile[:, ~bit] *= d0
            elif k == 6:
                ph = x["c"][0] + 1j * x["c"][1] if fl & 8 else 1.0  # phased: control = target = 1 after
                if fl & 1:
                    sel = ((bases >> q0) & 1).astype(bool)
                    sub = tile[sel]
                    _pair(sub, q1, _matrix({"kind": 4, "c": x["c"]}))
                    if fl & 8:
                        sub[:, ((lidx >> q1) & 1).astype(bool)] *= ph
                    tile[sel] = sub
                else:
                    src = lidx[(((lidx >> q0) & 1) == 1) & (((lidx >> q1) & 1) == 0)]
                    dst = src | (1 << q1)
                    tmp = tile[:, src].copy()
                    tile[:, src] = tile[:, dst]
                    tile[:, dst] = tmp * ph
            elif k == 7:
                nl, lmk = int(x["nl_mask"]), int(x["mask"])
                rows = (bases & nl) == nl
                cols = (lidx & lmk) == lmk
                tile[np.ix_(rows, cols)] *= -1
            else:
                raise AssertionError(f"unknown executor op {k}")
        psi[idx] = tile
    return psi
