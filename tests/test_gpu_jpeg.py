"""GPU parity of the baseline JPEG encoder: byte-identical to the reference's encoder (golden bytes
of jpeg_codec::process_encode_baseline) and to the oracle on full-size frames, through the host
and the device entry points, with the reference's status codes and capacity truncation."""
import json
import os

import numpy as np
import pytest

import imop_gb300 as I
from imop_gb300 import jpeg as J
from imop_gb300 import workloads
import oracle_py as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jpeg.npz")


def golden():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]))
    return [(c, z[f"img{c['image']}"], z[f"jpg{i}"]) for i, c in enumerate(meta["cases"])], meta["errors"]


CASES, ERRORS = golden()


@pytest.fixture(scope="module")
def enc():
    e = J.JpegEncoder()
    yield e
    e.close()


@pytest.mark.parametrize("case", CASES, ids=[c[0]["name"] for c in CASES])
def test_host_matches_golden(enc, case):
    c, img, want = case
    got = enc.encode(img, c["quality"], c["subsample"], c["cap"])
    assert got.size == want.size and np.array_equal(got, want)


@pytest.mark.parametrize("e", ERRORS, ids=[f"{e['w']}x{e['h']}_bd{e['bd']}_q{e['quality']}_{e['null_in']}{e['null_out']}"
                                           for e in ERRORS])
def test_status_codes_match_golden(enc, e):
    img = None if e["null_in"] else np.zeros((8, 8, 3), np.uint8)
    if e["null_out"]:
        import ctypes as C
        n = C.c_size_t(0)
        st = J._L().imop_jpeg_encode_host(enc.h, None if img is None else img.ctypes.data, e["w"], e["h"], e["bd"],
                                          e["quality"], 1, None, C.byref(n))
    else:
        st, _ = enc.encode_status(img, e["quality"], 1, bit_depth=e["bd"], width=e["w"], height=e["h"])
    assert st == e["status"]


def _frame(w, h, seed):
    """an ISP-like RGB8 frame: the oracle's output of a seeded raw scene"""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    f = rng.uniform(0.005, 0.05, 3).astype(np.float32)
    img = np.stack([127 + 110 * np.sin(f[c] * x + 0.8 * np.cos(f[2 - c] * y + c)) for c in range(3)], -1)
    img += rng.normal(0, 6, img.shape).astype(np.float32)
    return np.clip(img, 0, 255).astype(np.uint8)


@pytest.mark.parametrize("w,h", [(1006, 758), (4024, 3032), (1921, 1081)])
@pytest.mark.parametrize("ss", [0, 1, 2])
def test_full_size_matches_oracle(enc, w, h, ss):
    img = _frame(w, h, w + ss)
    q = (90, 75, 98)[ss]
    st, want = O.jpeg_encode(img, q, ss)
    assert st == 0
    got = enc.encode(img, q, ss)
    assert got.size == want.size and np.array_equal(got, want)


@pytest.mark.parametrize("q", [1, 5, 30, 50, 51, 99, 100])
def test_noise_every_quality_matches_oracle(enc, q):
    """high-entropy input: long codes, 0xFF bytes to stuff, ZRL runs at low quality"""
    rng = np.random.default_rng(q)
    img = rng.integers(0, 256, (517, 389, 3), dtype=np.uint8)
    st, want = O.jpeg_encode(img, q, q % 3)
    got = enc.encode(img, q, q % 3)
    assert np.array_equal(got, want)


def test_device_entry_point_and_reuse(enc):
    """device in / device out on a side stream, sizes on the device, truncation, and scratch
    reuse across frames of changing sizes (the cleared word stream)"""
    import torch
    dev = torch.device("cuda:0")
    s = torch.cuda.Stream()
    frames = [(_frame(640, 480, 1), 90, 1), (_frame(33, 27, 2), 50, 0), (_frame(1500, 900, 3), 95, 2),
              (_frame(640, 480, 1), 90, 1)]
    for img, q, ss in frames:
        h, w = img.shape[:2]
        st, want = O.jpeg_encode(img, q, ss)
        d_in = torch.from_numpy(img).to(dev)
        cap = J.max_bytes(w, h)
        d_out = torch.zeros(cap, dtype=torch.uint8, device=dev)
        d_size = torch.zeros(1, dtype=torch.int64, device=dev)
        torch.cuda.current_stream().synchronize()
        with torch.cuda.stream(s):
            enc.encode_device(d_in, w, h, d_out, cap, q, ss, d_size=d_size, stream=s.cuda_stream)
        total, written = enc.last_size()
        s.synchronize()
        assert total == written == want.size == int(d_size.item())
        assert np.array_equal(d_out[:written].cpu().numpy(), want)
    # truncation on the device: the first cap bytes, size = cap
    img, q, ss = frames[0]
    st, want = O.jpeg_encode(img, q, ss)
    for cap in (10, 623, 624, 5000):
        d_in = torch.from_numpy(img).to(dev)
        d_out = torch.full((cap + 64,), 0xAB, dtype=torch.uint8, device=dev)
        enc.encode_device(d_in, img.shape[1], img.shape[0], d_out, cap, q, ss)
        total, written = enc.last_size()
        assert total == want.size and written == cap
        out = d_out.cpu().numpy()
        assert np.array_equal(out[:cap], want[:cap]) and np.all(out[cap:] == 0xAB)


def test_isp_to_jpeg_on_device(enc):
    """the fused ISP's RGB8 output encoded where it lies: RAW -> JPEG without a host round trip"""
    import torch
    pl = workloads.c2_pipeline(1006, 758)
    raw = workloads.c2_frame(pl, 0)
    rgb_ref, _ = O.pipeline(pl, raw)
    st, want = O.jpeg_encode(rgb_ref.reshape(758, 1006, 3), 90, 1)
    isp = I.Isp(pl)
    d_raw = torch.from_numpy(np.ascontiguousarray(raw)).cuda()
    d_rgb = torch.empty((758, 1006, 3), dtype=torch.uint8, device="cuda")
    cap = J.max_bytes(1006, 758)
    d_out = torch.empty(cap, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    isp.run_device(d_raw, d_rgb, stream)
    enc.encode_device(d_rgb, 1006, 758, d_out, cap, 90, 1, stream=stream)
    total, written = enc.last_size()
    isp.close()
    assert written == want.size and np.array_equal(d_out[:written].cpu().numpy(), want)


def test_device_batch_matches_oracle(enc):
    """frames of different sizes, qualities and subsamplings on the two internal streams, with
    device size records; the caller's stream continues after the batch"""
    import torch
    specs = [(640, 480, 90, 1), (33, 27, 50, 0), (1500, 900, 95, 2), (1006, 758, 10, 1), (8, 8, 100, 0),
             (2000, 1000, 75, 2), (640, 480, 90, 1)]
    imgs = [_frame(w, h, 40 + k) for k, (w, h, q, ss) in enumerate(specs)]
    s = torch.cuda.Stream()
    d_in = [torch.from_numpy(im).cuda() for im in imgs]
    caps = [J.max_bytes(w, h) for (w, h, q, ss) in specs]
    d_out = [torch.full((c,), 0xAB, dtype=torch.uint8, device="cuda") for c in caps]
    d_size = torch.zeros(len(specs), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    frames = [(d_in[k], w, h, d_out[k], caps[k], q, ss, d_size[k:k + 1]) for k, (w, h, q, ss) in enumerate(specs)]
    with torch.cuda.stream(s):
        enc.encode_device_batch(frames, stream=s.cuda_stream)
        sizes = d_size.clone()  # ordered after the batch on the caller's stream
    s.synchronize()
    for k, (w, h, q, ss) in enumerate(specs):
        st, want = O.jpeg_encode(imgs[k], q, ss)
        n = int(sizes[k].item())
        assert n == want.size, k
        assert np.array_equal(d_out[k][:n].cpu().numpy(), want), k
    assert enc.last_size()[0] == int(sizes[-1].item())


def test_host_batch_matches_oracle(enc):
    """pinned and pageable host frames, an invalid frame in the middle (its own status, the others
    encoded), a truncating capacity"""
    import torch
    specs = [(640, 480, 90, 1), (1500, 900, 60, 0), (4, 4, 90, 1), (1006, 758, 85, 2), (333, 217, 30, 1)]
    frames, wants = [], []
    for k, (w, h, q, ss) in enumerate(specs):
        img = _frame(w, h, 70 + k)
        rgb = torch.from_numpy(img).pin_memory() if k % 2 == 0 else img
        cap = J.max_bytes(w, h) if k != 4 else 700
        out = np.zeros(cap, np.uint8)
        frames.append((rgb, q, ss, out))
        wants.append(O.jpeg_encode(img, q, ss, cap) if (w >= 8 and h >= 8) else (J.IMAGE_TOO_SMALL, None))
    res = enc.encode_host_batch(frames)
    for k, ((st, n), (wst, want)) in enumerate(zip(res, wants)):
        assert st == wst, k
        if st == 0:
            assert n == want.size and np.array_equal(frames[k][3][:n], want), k


def test_device_then_host_calls_without_sync(enc):
    """a device encode on the caller's stream followed at once by host encodes on the same
    context: the context orders the uses of its scratch across streams"""
    import torch
    big = _frame(3000, 2000, 5)
    small = _frame(640, 480, 6)
    st_big, want_big = O.jpeg_encode(big, 90, 1)
    st_small, want_small = O.jpeg_encode(small, 80, 0)
    s = torch.cuda.Stream()
    d_in = torch.from_numpy(big).cuda()
    cap = J.max_bytes(3000, 2000)
    d_out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        enc.encode_device(d_in, 3000, 2000, d_out, cap, 90, 1, stream=s.cuda_stream)
        got = enc.encode(small, 80, 0)  # no synchronisation with s in between
        assert np.array_equal(got, want_small)
    s.synchronize()
    assert np.array_equal(d_out[:want_big.size].cpu().numpy(), want_big)


@pytest.mark.parametrize("kind", ["noise_8k_q100_444", "q1", "flat0", "flat255", "spike", "stripes_odd"])
def test_extremes_match_oracle(enc, kind):
    """the bit-stream capacity bound at full load (8K noise at quality 100, 4:4:4: about 250 MB of
    output), all-zero AC blocks (quality 1), flat frames, a lone bright pixel, and odd sizes with
    one-pixel stripes (runs of 16 zeros and long codes)"""
    rng = np.random.default_rng(len(kind))
    if kind == "noise_8k_q100_444":
        img, q, ss = rng.integers(0, 256, (4320, 7680, 3), dtype=np.uint8), 100, 0
    elif kind == "q1":
        img, q, ss = _frame(1001, 777, 3), 1, 1
    elif kind in ("flat0", "flat255"):
        img, q, ss = np.full((64, 80, 3), 0 if kind == "flat0" else 255, np.uint8), 90, 2
    elif kind == "spike":
        img = np.zeros((48, 48, 3), np.uint8)
        img[21, 30] = (255, 255, 255)
        q, ss = 100, 1
    else:
        img = np.zeros((259, 333, 3), np.uint8)
        img[:, ::2] = 255
        img[::3, :, 1] = 17
        q, ss = 97, 0
    st, want = O.jpeg_encode(img, q, ss)
    assert st == 0
    got = enc.encode(img, q, ss)
    assert got.size == want.size and np.array_equal(got, want)
