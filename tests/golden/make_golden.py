"""Regenerates the golden fixtures in this folder from the SyFrack source tree.

Run in a checkout that has the reference next to it:
    python tests/golden/make_golden.py /path/to/SyFrack
It reads, as data:
  crates/syfrack-core/tests/fixtures/parity/{sphere,mandelbulb,mandelbox,menger}.ron
      -> de_parity_<name>.json  (64 LCG points, distance, traps, iterations;
         the samples graph_parity.rs checks the bundled graphs against)
  graphs/{sphere,mandelbulb,mandelbox,menger}.ron
      -> graph_<name>.json      (nodes, links, safety, bounding_radius_hint)
  scenes/{mandelbox,menger,mandelbulb}.ron
      -> scene_<name>.json      (the scene file as JSON: graph, camera, lights, material)
  scenes/{eclosion-brume,puits-des-eons}.ron, scenes/showcase/la-cathedrale-des-marees-neons.ron,
  scenes/studies/cathedrale-des-marees-20261020/etude-neons.ron
      -> scene_<name>.json      (the same, for the reader's material, light and fog
         fields: finishes with details, projectors and tubes, a texture graph; 14
         and 82 lights, past the descriptor's inline eight)
  crates/syfrack-render/tests/fixtures/parity/{mandelbox,menger,mandelbulb}.exr
      -> film_<name>_blocks.json (the reference's own 640x360, 64-spp render of that
         scene, reduced to what the film gate reads: 8x8 block means of the 8-bit
         AgX + sRGB development of the image, per channel, and the image's channel
         means in linear and in 8-bit)
The JSON files are committed; nothing at test time reads the reference.
"""
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from syfrack_gb300 import ron  # noqa: E402

NAMES = ["sphere", "mandelbulb", "mandelbox", "menger"]
EXTENTS = {"sphere": 3.0, "mandelbulb": 1.6, "mandelbox": 8.0, "menger": 1.6}


def to_json(v):
    if isinstance(v, ron.Unit):
        return v.name
    if isinstance(v, ron.Tuple) and v.name:  # Kelvin(5500.0), Graph((...)): keep the name
        return {"__name__": v.name, "__items__": [to_json(x) for x in v.items]}
    if isinstance(v, ron.Tuple):
        return [to_json(x) for x in v.items]
    if isinstance(v, dict):
        return {k: to_json(x) for k, x in v.items()}
    if isinstance(v, list):
        return [to_json(x) for x in v]
    return v


SCENES = ["mandelbox", "menger", "mandelbulb"]
# scene files without a reference render (paths under scenes/; fixtures named by the file)
EXTRA_SCENES = ["eclosion-brume", "puits-des-eons", "showcase/la-cathedrale-des-marees-neons",
                "studies/cathedrale-des-marees-20261020/etude-neons"]


def read_exr(path):
    """A scanline-free OpenEXR reader for the fixtures' layout: tiled, one level,
    FLOAT channels, RLE or no compression (OpenEXR's byte predictor and
    interleave). Returns (image[h, w, channels], channel names)."""
    d = open(path, "rb").read()
    assert d[:4] == b"\x76\x2f\x31\x01", "not an OpenEXR file"
    pos, hdr = 8, {}
    while True:
        end = d.index(b"\0", pos)
        name = d[pos:end].decode()
        pos = end + 1
        if not name:
            break
        end = d.index(b"\0", pos)
        pos = end + 1
        size = struct.unpack("<I", d[pos:pos + 4])[0]
        pos += 4
        hdr[name] = d[pos:pos + size]
        pos += size
    chans, v, p = [], hdr["channels"], 0
    while v[p] != 0:
        e = v.index(b"\0", p)
        chans.append(v[p:e].decode())
        p = e + 1
        assert struct.unpack("<i", v[p:p + 4])[0] == 2, "FLOAT channels only"
        p += 16
    comp = hdr["compression"][0]
    x0, y0, x1, y1 = struct.unpack("<4i", hdr["dataWindow"])
    W, H = x1 - x0 + 1, y1 - y0 + 1
    tw, th, _ = struct.unpack("<IIB", hdr["tiles"])
    ntx, nty = (W + tw - 1) // tw, (H + th - 1) // th
    offs = struct.unpack(f"<{ntx * nty}Q", d[pos:pos + 8 * ntx * nty])
    img = np.zeros((H, W, len(chans)), np.float32)
    for off in offs:
        tx, ty, _, _, size = struct.unpack("<5i", d[off:off + 20])
        data = d[off + 20:off + 20 + size]
        w, h = min(tw, W - tx * tw), min(th, H - ty * th)
        if size < w * h * len(chans) * 4:
            assert comp == 1, "RLE or uncompressed tiles only"
            out, i = bytearray(), 0
            while i < len(data):
                c = struct.unpack("b", data[i:i + 1])[0]
                i += 1
                if c < 0:
                    out += data[i:i - c]
                    i -= c
                else:
                    out += bytes([data[i]]) * (c + 1)
                    i += 1
            acc = bytearray(len(out))
            run = out[0]
            acc[0] = run
            for k in range(1, len(out)):
                run = (run + out[k] - 128) & 0xFF
                acc[k] = run
            half = (len(acc) + 1) // 2
            raw = bytearray(len(acc))
            raw[0::2] = acc[:half]
            raw[1::2] = acc[half:]
            data = bytes(raw)
        tile = np.frombuffer(data, np.float32).reshape(h, len(chans), w)
        img[ty * th:ty * th + h, tx * tw:tx * tw + w, :] = tile.transpose(0, 2, 1)
    return img, chans


# AgX (Troy Sobotka) with Benjamin Wrensch's polynomial fit of its sigmoid: the
# classic scenes' tone map (Tonemap::Agx{slope 1, power 1, offset 0}); their other
# look steps (exposure 0, 6500 K balance, zero grades, saturation 1) are identities.
AGX_IN = np.array([[0.84247906, 0.0784336, 0.079223745], [0.04232824, 0.87846864, 0.07916613],
                   [0.042375655, 0.0784336, 0.879143]])
AGX_OUT = np.array([[1.196879, -0.09802088, -0.09902974], [-0.05289685, 1.1519031, -0.09896118],
                    [-0.052971635, -0.09804345, 1.1510737]])
AGX_MIN_EV, AGX_MAX_EV = -12.473934, 4.026069


def develop8(rgb):
    """The film gate's display transform: AgX to display-linear, sRGB encode, 8 bits
    (rounded; the reference also dithers, which moves block means by < 0.5/64)."""
    v = np.maximum(rgb.astype(np.float64), 1e-10) @ AGX_IN.T
    v = np.clip((np.log2(np.maximum(v, 1e-300)) - AGX_MIN_EV) / (AGX_MAX_EV - AGX_MIN_EV), 0.0, 1.0)
    x2 = v * v
    x4 = x2 * x2
    v = 15.5 * x4 * x2 - 40.14 * x4 * v + 31.96 * x4 - 6.868 * x2 * v + 0.4298 * x2 + 0.1191 * v - 0.00232
    v = np.maximum(v, 0.0) @ AGX_OUT.T
    x = np.power(np.clip(v, 0.0, 1.0), 2.2)
    e = np.where(x <= 0.0031308, 12.92 * x, 1.055 * np.power(x, 1.0 / 2.4) - 0.055)
    return np.floor(e * 255.0 + 0.5)


def block_means(img8, b=8):
    h, w, _ = img8.shape
    out = np.zeros(((h + b - 1) // b, (w + b - 1) // b, 3))
    for by in range(out.shape[0]):
        for bx in range(out.shape[1]):
            out[by, bx] = img8[by * b:(by + 1) * b, bx * b:(bx + 1) * b].reshape(-1, 3).mean(0)
    return out


def main(root):
    for name in NAMES:
        fx = ron.load(os.path.join(root, "crates/syfrack-core/tests/fixtures/parity", f"{name}.ron"))
        rows = [{"p": ron.vec(r["p"]), "distance": r["distance"], "traps": ron.vec(r["traps"]),
                 "iterations": r["iterations"]} for r in fx]
        with open(os.path.join(HERE, f"de_parity_{name}.json"), "w") as f:
            json.dump({"source": f"crates/syfrack-core/tests/fixtures/parity/{name}.ron",
                       "extent": EXTENTS[name], "lcg_seed": 11, "samples": rows}, f, indent=0)
        g = ron.load(os.path.join(root, "graphs", f"{name}.ron"))
        with open(os.path.join(HERE, f"graph_{name}.json"), "w") as f:
            json.dump({"source": f"graphs/{name}.ron", "graph": to_json(g)}, f, indent=1)
    for name in SCENES:
        v = ron.load(os.path.join(root, "scenes", f"{name}.ron"))
        with open(os.path.join(HERE, f"scene_{name}.json"), "w") as f:
            json.dump({"source": f"scenes/{name}.ron", "scene": to_json(v)}, f, indent=0)
        img, chans = read_exr(os.path.join(root, "crates/syfrack-render/tests/fixtures/parity", f"{name}.exr"))
        rgb = img[..., [chans.index("R"), chans.index("G"), chans.index("B")]]
        enc = develop8(rgb)
        bm = block_means(enc)
        with open(os.path.join(HERE, f"film_{name}_blocks.json"), "w") as f:
            json.dump({"source": f"crates/syfrack-render/tests/fixtures/parity/{name}.exr",
                       "render": {"width": 640, "height": 360, "spp": 64, "max_bounces": 4, "max_steps": 256},
                       "blocks": [[round(float(x), 3) for x in row.reshape(-1)] for row in bm],
                       "mean_linear": [float(x) for x in rgb.reshape(-1, 3).mean(0)],
                       "mean_8bit": [float(x) for x in enc.reshape(-1, 3).mean(0)]}, f)
    for name in EXTRA_SCENES:
        v = ron.load(os.path.join(root, "scenes", f"{name}.ron"))
        with open(os.path.join(HERE, f"scene_{os.path.basename(name)}.json"), "w") as f:
            json.dump({"source": f"scenes/{name}.ron", "scene": to_json(v)}, f, indent=0)
    print("wrote", len(NAMES) * 2 + len(SCENES) * 2 + len(EXTRA_SCENES), "files")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
