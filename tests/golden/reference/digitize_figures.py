"""Read the curves of three figures of Caracal's manual into text fixtures.

Caracal ships no numeric outputs for its examples, but its manual plots
three: the IRC of the ANA_CH4OH surface from examples/explore/ts_irc_ch4oh
(manual/figures/irc_ch4oh.png) and the H + H2 PMF and transmission
coefficient of examples/calc_rate/h+h2 at 300 K (pmf_h3.png,
kappa_h3.png).  This script decodes those PNG files (8-bit RGB(A),
non-interlaced; the decoder below undoes PNG's five scanline filters),
takes the centre row of the plotted line in every pixel column, maps
pixels to data by the axis tick marks found in the image, and writes

  figure_irc_ch4oh.txt   s (bohr amu^1/2), E (Hartree), half line width (Hartree)
  figure_pmf_h3.txt      xi, PMF (kJ/mol), half line width (kJ/mol)
  figure_kappa_h3.txt    t (fs), kappa, half line width

The tick positions are listed in each file's header.  The reading error
of a point is about one pixel in each direction (1/16000 Hartree,
1/20 kJ/mol and 1/4000 in kappa vertically).

Run: python tests/golden/reference/digitize_figures.py [path of the Caracal tree]
"""
import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_png(path):
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
    if depth != 8 or interlace != 0 or ctype not in (2, 6):
        raise ValueError(f"{path}: only 8-bit non-interlaced RGB/RGBA is read here")
    ch = 3 if ctype == 2 else 4
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)
    stride = w * ch
    out = np.zeros((h, stride), np.int64)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)].astype(np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, np.int64)
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                c = prev[x - ch] if x >= ch else 0
                b = prev[x]
                if f == 1:
                    pr = a
                elif f == 3:
                    pr = (a + b) // 2
                else:                               # Paeth
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch)


def _runs(idx):
    """Centres of runs of consecutive integers."""
    out, start = [], None
    for i, v in enumerate(idx):
        if start is None:
            start = v
        if i + 1 == len(idx) or idx[i + 1] != v + 1:
            out.append(0.5 * (start + v))
            start = None
    return out


def _run_bounds(idx):
    """(first, last) of each run of consecutive integers."""
    out, start = [], None
    for i, v in enumerate(idx):
        if start is None:
            start = v
        if i + 1 == len(idx) or idx[i + 1] != v + 1:
            out.append((start, v))
            start = None
    return out


def digitize(path, xticks, yticks):
    """xticks / yticks: the data values of the labelled tick marks, in
    order; their pixel positions are found on the frame."""
    im = read_png(path)
    r, g, b = im[..., 0], im[..., 1], im[..., 2]
    a = im[..., 3] if im.shape[2] == 4 else np.full_like(r, 255)
    dark = (r < 80) & (g < 80) & (b < 80) & (a > 128)
    line = (r > 100) & (r < 200) & (g < 60) & (b > 180) & (a > 128)
    cols = dark.sum(axis=0)
    rows = dark.sum(axis=1)
    half_w, half_h = im.shape[1] // 2, im.shape[0] // 2
    left = int(np.argmax(cols[:half_w]))
    right = half_w + int(np.argmax(cols[half_w:]))
    top = int(np.argmax(rows[:half_h]))
    bottom = half_h + int(np.argmax(rows[half_h:]))
    # gnuplot mirrors the tick marks on the top and right frames, where the
    # curves of these figures do not cross them
    ty = _runs([y for y in range(im.shape[0]) if dark[y, right - 10:right - 3].sum() >= 6])
    tx = _runs([x for x in range(left - 3, right + 4) if dark[top + 4:top + 10, x].sum() >= 5])
    if len(ty) != len(yticks) or len(tx) != len(xticks):
        raise ValueError(f"{path}: found {len(tx)} x and {len(ty)} y ticks")
    fy = np.polyfit(ty, yticks[::-1], 1)        # pixel rows grow downwards
    fx = np.polyfit(tx, xticks, 1)
    # the key's sample line: the longest horizontal run of the line colour
    # in the top sixth of the plot; blank its box out
    best = (0, 0, 0, 0)
    for y in range(top, top + (bottom - top) // 6):
        xs = np.nonzero(line[y])[0]
        for x0 in _run_bounds(xs):
            if x0[1] - x0[0] > best[2] - best[1]:
                best = (y, x0[0], x0[1], 0)
    if best[2] - best[1] > 60:
        line[best[0] - 4:best[0] + 5, best[1] - 2:best[2] + 3] = False
    pts = []
    for x in range(left + 2, right - 1):
        ys = np.nonzero(line[top + 2:bottom - 2, x])[0] + top + 2
        if len(ys) == 0:
            continue
        pts.append((np.polyval(fx, x), np.polyval(fy, 0.5 * (ys.min() + ys.max())),
                    0.5 * abs(fy[0]) * (ys.max() - ys.min() + 1)))
    return np.array(pts), tx, ty


def main(tree="/root/reference"):
    figs = {
        "irc_ch4oh": (np.arange(-2.5, 2.01, 0.5), np.arange(-0.74, -0.6999, 0.005)),
        "pmf_h3": (np.arange(-0.2, 1.201, 0.2), np.arange(0.0, 50.01, 5.0)),
        "kappa_h3": (np.arange(0.0, 50.01, 5.0), np.arange(0.75, 1.0001, 0.05)),
    }
    heads = {"irc_ch4oh": "s (bohr amu^1/2)  E (Hartree)  half width (Hartree)",
             "pmf_h3": "xi  PMF (kJ/mol)  half width (kJ/mol)",
             "kappa_h3": "t (fs)  kappa  half width"}
    for name, (xt, yt) in figs.items():
        src = os.path.join(tree, "manual", "figures", name + ".png")
        pts, tx, ty = digitize(src, xt, yt)
        with open(os.path.join(HERE, f"figure_{name}.txt"), "w") as fh:
            fh.write(f"# digitised from Caracal's manual/figures/{name}.png by digitize_figures.py\n")
            fh.write(f"# x ticks {[round(float(v), 4) for v in xt]} at pixels {tx}\n")
            fh.write(f"# y ticks {[round(float(v), 4) for v in yt]} at pixels {ty}\n")
            fh.write(f"# {heads[name]}\n")
            for p in pts:
                fh.write(f"{p[0]:.6f} {p[1]:.7f} {p[2]:.7f}\n")
        print(name, len(pts))


if __name__ == "__main__":
    main(*sys.argv[1:])
