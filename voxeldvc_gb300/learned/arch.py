"""Architecture of the learned initial guess (pure data, no device code).

Input: f and g low-passed and sampled every 4 voxels, 2 channels, grid G.
Output: the displacement (3 channels, voxels) on the stride-8 voxel grid
n = (G - 1) // 2 + 1, which is the node grid of an h = 8 mesh.

    c1  2 -> 16, stride 1   grid G        ReLU
    c2 16 -> 32, stride 2   G -> n        ReLU
    c3 32 -> 32, stride 1   n             ReLU   (also the skip branch)
    c4 32 -> 32, stride 2   n -> m        ReLU
    c5 32 -> 32, stride 1   m             ReLU
    c6 32 -> 32, stride 1   m             ReLU
    up  linear 2x           m -> n, concatenated as [up(c6) | c3] (64 ch)
    c7 64 -> 16, stride 1   n             ReLU
    c8 16 ->  3, stride 1   n             (linear, FP32 output)

All convolutions are 3x3x3 with zero padding.  Receptive field of an
output: about 41 input samples (~160 voxels) per axis.
"""
LAYERS = (
    dict(name="c1", cin=2, cout=16, stride=1, relu=True),
    dict(name="c2", cin=16, cout=32, stride=2, relu=True),
    dict(name="c3", cin=32, cout=32, stride=1, relu=True),
    dict(name="c4", cin=32, cout=32, stride=2, relu=True),
    dict(name="c5", cin=32, cout=32, stride=1, relu=True),
    dict(name="c6", cin=32, cout=32, stride=1, relu=True),
    dict(name="c7", cin=64, cout=16, stride=1, relu=True),
    dict(name="c8", cin=16, cout=3, stride=1, relu=False),
)
LAYER = {l["name"]: l for l in LAYERS}
OUT_STRIDE = 8   # voxels between output samples
IN_STRIDE = 4    # voxels between input samples


def grids(G):
    """(G, n, m) per axis for an input grid G (tuple of 3)."""
    n = tuple((g - 1) // 2 + 1 for g in G)
    m = tuple((k - 1) // 2 + 1 for k in n)
    return tuple(G), n, m


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
