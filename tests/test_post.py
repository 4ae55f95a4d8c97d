"""The presentation pass (post_proc.frag:16-44 as grisPostProcess) and the headless PNG writer:
the oracle's pass against the reference's own post_proc.frag compiled as C++ (oracle/_ref,
byte for byte) and against a float64 numpy restatement of the shader (tone curves, gamma,
composition flags, the fragment shader's texel mapping), the library's PNG files decoded with
zlib, and on the GPU the kernel against the oracle bit for bit (colour and bytes)."""
import os
import struct
import zlib

import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O


def _images(W, H, seed):
    rng = np.random.default_rng(seed)
    d = rng.exponential(0.6, size=(W * H, 4)).astype(np.float32)
    i = rng.exponential(0.3, size=(W * H, 4)).astype(np.float32)
    d[::97, 0] = 0.0
    i[::89, 1] = 50.0          # very bright
    d[5, :3] = np.nan          # NaN radiance ends as 0 in the bytes
    return d, i


def _numpy_post(W, H, d, i, st):
    x = np.arange(W)
    y = np.arange(H)
    cx = ((W - 1) * ((x + 0.5) / W)).astype(np.int64)
    cy = ((H - 1) * ((y + 0.5) / H)).astype(np.int64)
    src = (cy[:, None] * W + cx[None, :]).reshape(-1)
    c = np.zeros((W * H, 3))
    if not st.noDirect:
        c = c + d[src, :3].astype(np.float64)
    if not st.noIndirect:
        c = c + i[src, :3].astype(np.float64)

    def curve(v):
        return (v * (v * 0.22 + 0.03) + 0.002) / (v * (v * 0.22 + 0.3) + 0.06) - 1.0 / 30.0
    if st.toneMapping == 1:
        c = curve(c * 1.6) / curve(11.2)
    elif st.toneMapping == 2:
        c = (c * (c * 2.51 + 0.03)) / (c * (c * 2.43 + 0.59) + 0.14)
    if st.correctGamma:
        with np.errstate(invalid="ignore"):
            c = np.where(c >= 0, np.power(np.maximum(c, 0), 1 / 2.2), np.nan)
    return c


SETTINGS = [dict(), dict(toneMapping=G.TONEMAP_NONE), dict(toneMapping=G.TONEMAP_ACES),
            dict(correctGamma=False), dict(noDirect=True), dict(noIndirect=True, toneMapping=G.TONEMAP_ACES)]


@pytest.mark.parametrize("kw", SETTINGS, ids=["defaults", "none", "aces", "no_gamma", "no_direct", "aces_no_indirect"])
def test_oracle_post_matches_numpy(kw):
    W, H = 37, 23
    d, i = _images(W, H, 3)
    st = G.PostSettings.make(**kw)
    color, rgba = O.post_process(W, H, d, i, st)
    want = _numpy_post(W, H, d, i, st)
    ok = np.isfinite(want)
    assert np.array_equal(ok, np.isfinite(color[:, :3]))
    np.testing.assert_allclose(color[:, :3][ok], want[ok], rtol=3e-5, atol=1e-6)
    assert np.all(color[:, 3] == 1.0) and np.all(rgba[:, 3] == 255)
    wb = np.where(ok, np.clip(np.nan_to_num(want, nan=0.0), 0, 1) * 255.0, 0.0)
    assert np.abs(rgba[:, :3].astype(np.float64) - wb).max() <= 0.5 + 1e-3
    assert np.all(rgba[5, :3] == 0) or kw.get("noDirect")


@pytest.mark.parametrize("kw", SETTINGS, ids=["defaults", "none", "aces", "no_gamma", "no_direct", "aces_no_indirect"])
@pytest.mark.parametrize("size", [(37, 23), (64, 1), (1, 9), (130, 77)], ids=["37x23", "64x1", "1x9", "130x77"])
def test_oracle_post_matches_compiled_reference(kw, size):
    """The oracle's presentation pass against post_proc.frag itself (compiled as C++ by
    oracle/ref/make_ref.py, run per fragment of the full-screen quad): the fragment colours
    (NaN channels as the canonical quiet NaN) and their UNORM8 bytes, byte for byte, over images
    with zeros, very bright texels, NaN radiance and odd sizes (texel mapping ivec2((size-1) uv))."""
    if not os.path.exists(O.POST_REF_LIB):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    W, H = size
    d, i = _images(W, H, 7 + W)
    st = G.PostSettings.make(**kw)
    color, rgba = O.post_process(W, H, d, i, st)
    ref_color, ref_rgba = O.post_process(W, H, d, i, st, reference=True)
    assert color.tobytes() == ref_color.tobytes()
    assert rgba.tobytes() == ref_rgba.tobytes()


def test_png_writer_roundtrip(tmp_path):
    W, H = 301, 7   # more than one stored block per image (7 x 1205 B rows > 0; 301*4+1 per row)
    rng = np.random.default_rng(1)
    rgba = rng.integers(0, 256, size=(W * H, 4), dtype=np.uint8)
    p = tmp_path / "a.png"
    G.write_png(str(p), rgba, W, H)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        chunks.append((typ, body))
        pos += 12 + n
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[0][1][:10])
    assert (w, h, depth, ctype) == (W, H, 8, 6)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, np.uint8).reshape(H, W * 4 + 1)
    assert np.all(rows[:, 0] == 0)
    assert rows[:, 1:].tobytes() == rgba.tobytes()
    big = np.zeros((400 * 50, 4), np.uint8)   # 80 kB of rows: two stored blocks
    G.write_png(str(tmp_path / "b.png"), big, 400, 50)
    with pytest.raises(G.GrisError):
        G.write_png(str(tmp_path / "missing_dir" / "c.png"), big, 400, 50)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", SETTINGS, ids=["defaults", "none", "aces", "no_gamma", "no_direct", "aces_no_indirect"])
def test_gpu_post_matches_oracle(kw):
    import torch
    W, H = 1920 + 7, 131
    d, i = _images(W, H, 5)
    st = G.PostSettings.make(**kw)
    want_c, want_b = O.post_process(W, H, d, i, st)
    ctx = G.Context(0)
    dd = torch.from_numpy(d).cuda()
    di = torch.from_numpy(i).cuda()
    col = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    byt = torch.zeros((W * H, 4), dtype=torch.uint8, device="cuda")
    b = G.PostBindings(W, H, dd.data_ptr(), di.data_ptr(), col.data_ptr(), byt.data_ptr())
    ctx.post_process(b, st)
    ctx.sync()
    assert col.cpu().numpy().tobytes() == want_c.tobytes()
    assert byt.cpu().numpy().tobytes() == want_b.tobytes()
    ctx.close()


@pytest.mark.gpu
def test_gpu_frame_to_png(tmp_path):
    """A rendered frame (direct + indirect) through the presentation pass into a PNG file."""
    import torch
    hs = G.HostScene(0, seed=2)
    W, H = 64, 48
    cams, prevs = G.sequence_cameras(hs, 2, W, H, seed=3)
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    for f in range(2):
        fr.render_di(scene, cams[f], prevs[f], G.DISettings.make(temporalReuse=True), G.Settings.make(maxDepth=4))
    dptr, _ = fr.device_ptr(G.BUF_DIRECT_OUTPUT)
    iptr, _ = fr.device_ptr(G.BUF_OUTPUT)
    byt = torch.zeros((W * H, 4), dtype=torch.uint8, device="cuda")
    ctx.post_process(G.PostBindings(W, H, dptr, iptr, 0, byt.data_ptr()), G.PostSettings.make())
    ctx.sync()
    want_c, want_b = O.post_process(W, H, fr.download(G.BUF_DIRECT_OUTPUT), fr.download(G.BUF_OUTPUT),
                                    G.PostSettings.make())
    got = byt.cpu().numpy()
    assert got.tobytes() == want_b.tobytes()
    assert got[:, :3].max() > 0
    G.write_png(str(tmp_path / "frame.png"), got, W, H)
    assert (tmp_path / "frame.png").stat().st_size > W * H * 4
    fr.close(); scene.close(); ctx.close()
