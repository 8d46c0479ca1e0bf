"""Independent pure-Python restatements of the integer parts of Lumen's shader utilities, used to pin the
C oracle with known answers: pcg4d / rand (src/shaders/utils.glsl:121-148) and offset_ray (utils.glsl:73-84).
"""
import struct

M32 = 0xFFFFFFFF


def pcg4d(v):
    x, y, z, w = [(c * 1664525 + 1013904223) & M32 for c in v]
    x = (x + y * w) & M32
    y = (y + z * x) & M32
    z = (z + x * y) & M32
    w = (w + y * z) & M32
    x ^= x >> 16
    y ^= y >> 16
    z ^= z >> 16
    w ^= w >> 16
    x = (x + y * w) & M32
    y = (y + z * x) & M32
    z = (z + x * y) & M32
    w = (w + y * z) & M32
    return [x, y, z, w]


def f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def uint_to_float(x):
    return f32(struct.unpack("<f", struct.pack("<I", 0x3F800000 | (x >> 9)))[0] - 1.0)


def rand_stream(x, y, frame, n):
    """The first n draws of rand() for seed (x, y, frame, 0)."""
    s = [x, y, frame, 0]
    out = []
    for _ in range(n):
        s[3] = (s[3] + 1) & M32
        out.append(uint_to_float(pcg4d(s)[0]))
    return out


def offset_ray(p, n):
    def bits(f):
        return struct.unpack("<i", struct.pack("<f", f))[0]

    def unbits(i):
        return struct.unpack("<f", struct.pack("<i", i))[0]

    out = []
    for pc, nc in zip(p, n):
        pc, nc = f32(pc), f32(nc)
        of = int(f32(256.0 * nc))  # float product rounded to FP32, then truncated like GLSL int()
        moved = unbits(bits(pc) + (-of if pc < 0 else of))
        out.append(f32(pc + f32(f32(1.0 / 65536.0) * nc)) if abs(pc) < 1.0 / 32.0 else moved)
    return out
