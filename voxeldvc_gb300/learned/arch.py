"""Architecture of the learned initial guess (pure data, no device code).

A 4-level 3-D convolutional encoder-decoder with 32 base channels.  Input:
f and g low-passed and sampled every 4 voxels (2 channels, grid G0 -- 129^3
for a 513^3 pair).  Output: the displacement (3 channels, voxels) on the
stride-8 voxel grid G1 = (G0 - 1) // 2 + 1, which is the node grid of an
h = 8 mesh.  Grids: G(k+1) = (G(k) - 1) // 2 + 1.

    level  grid        encoder                                decoder
    0      G0 (129^3)  e1   2 ->  32 s1
    1      G1 ( 65^3)  e2a  32 ->  64 s2, e2b  64 ->  64      d2  (64 up + 64 skip) -> 32, out 32 -> 3
    2      G2 ( 33^3)  e3a  64 -> 128 s2, e3b 128 -> 128      d3  (128 up + 128 skip) -> 64
    3      G3 ( 17^3)  e4a 128 -> 128 s2, e4b 128 -> 128

Every convolution is 3x3x3 with zero padding and ReLU except `out`
(linear, FP32 output).  The decoder upsamples linearly by 2 and
concatenates [upsampled | skip] channels.  About 2.27M parameters.
"""
LAYERS = (
    dict(name="e1", cin=2, cout=32, stride=1, relu=True),
    dict(name="e2a", cin=32, cout=64, stride=2, relu=True),
    dict(name="e2b", cin=64, cout=64, stride=1, relu=True),
    dict(name="e3a", cin=64, cout=128, stride=2, relu=True),
    dict(name="e3b", cin=128, cout=128, stride=1, relu=True),
    dict(name="e4a", cin=128, cout=128, stride=2, relu=True),
    dict(name="e4b", cin=128, cout=128, stride=1, relu=True),
    dict(name="d3", cin=256, cout=64, stride=1, relu=True),
    dict(name="d2", cin=128, cout=32, stride=1, relu=True),
    dict(name="out", cin=32, cout=3, stride=1, relu=False),
)
LAYER = {l["name"]: l for l in LAYERS}
OUT_STRIDE = 8   # voxels between output samples
IN_STRIDE = 4    # voxels between input samples
LEVELS = 4


def grids(G):
    """(G0, G1, G2, G3) per axis for an input grid G (tuple of 3)."""
    out = [tuple(int(g) for g in G)]
    for _ in range(LEVELS - 1):
        out.append(tuple((k - 1) // 2 + 1 for k in out[-1]))
    return tuple(out)


def input_grid(shape):
    """Input grid of a volume of `shape` voxels (x, y, z)."""
    return tuple((s - 1) // IN_STRIDE + 1 for s in shape)


def param_layout():
    """[(name, w_offset, w_size, b_offset, n_out, cin)] in the flat FP32
    parameter vector (weights [n_out][27][cin] then bias [n_out], per layer)."""
    out, off = [], 0
    for l in LAYERS:
        ws = l["cout"] * 27 * l["cin"]
        out.append((l["name"], off, ws, off + ws, l["cout"], l["cin"]))
        off += ws + l["cout"]
    return out, off
