"""enblend's nearest-feature seam mask on the GPU (enb_nft_mask) against the
reference's own masks (tests/golden/reference_nft.npz, from src/nearest.h
compiled unmodified) and against the oracle on random footprints, the
benchmark canvas and with wrap-around, bit for bit; the overlap rejection;
host buffers; the mask driving enb_enblend; and enbgpu-enblend generating
its seams with --fine-mask --no-optimize."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NGOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "reference_nft.npz")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("k", range(int(NGOLDEN["nft_count"])))
def test_nft_mask_against_reference(ctx, k):
    import enbgpu
    wa, ba, wrap = NGOLDEN[f"nft{k}_white"], NGOLDEN[f"nft{k}_black"], bool(int(NGOLDEN[f"nft{k}_wrap"]))
    want = NGOLDEN[f"nft{k}_mask"]
    if want.size == 0:
        with pytest.raises(enbgpu.EnbError):
            ctx.nft_mask(_dev(wa), _dev(ba), wrap=wrap)
        return
    assert np.array_equal(ctx.nft_mask(_dev(wa), _dev(ba), wrap=wrap).cpu().numpy(), want)


@pytest.mark.parametrize("wrap", [False, True])
@pytest.mark.parametrize("seed", range(4))
def test_nft_mask_random_against_oracle(ctx, orc, wrap, seed):
    rng = np.random.default_rng(700 + seed)
    for _ in range(6):
        h, w = int(rng.integers(2, 300)), int(rng.integers(2, 500))
        wa = np.where(rng.random((h, w)) < rng.uniform(0.2, 0.9), 255, 0).astype(np.uint8)
        ba = np.where(rng.random((h, w)) < rng.uniform(0.2, 0.9), 255, 0).astype(np.uint8)
        try:
            want = orc.nft_mask(wa, ba, wrap)
        except ValueError:
            import enbgpu
            with pytest.raises(enbgpu.EnbError):
                ctx.nft_mask(_dev(wa), _dev(ba), wrap=wrap)
            continue
        got = ctx.nft_mask(_dev(wa), _dev(ba), wrap=wrap).cpu().numpy()
        assert np.array_equal(got, want), (h, w)
        # host buffers give the same mask
        assert np.array_equal(ctx.nft_mask(wa, ba, wrap=wrap), want)


@pytest.mark.parametrize("wrap", [False, True])
def test_nft_mask_benchmark_canvas(ctx, orc, wrap):
    """The footprints of the enblend benchmark: 2 x 4096x3072 offset by 2867
    on the 6963x3072 canvas."""
    from enbgpu import synthetic
    white, black, _ = synthetic.panorama_pair(3072, 4096, 2867, np.uint16, seed=2)
    wa, ba = orc.alpha_of(white), orc.alpha_of(black)
    want = orc.nft_mask(wa, ba, wrap)
    got = ctx.nft_mask(_dev(wa), _dev(ba), wrap=wrap).cpu().numpy()
    assert np.array_equal(got, want)
    if not wrap:
        # a seam through the overlap: the black image (left, columns 0..4095)
        # keeps its own part, the white one (right, from column 2867) its own
        # (with wrap the canvas's right end also neighbours the left one)
        assert want[:, :2867].max() == 0 and want[:, 4096:].min() == 255


def test_nft_mask_drives_enblend(ctx, orc):
    from enbgpu import synthetic
    white, black, _ = synthetic.panorama_pair(300, 400, 260, np.uint16, seed=5)
    wa, ba = orc.alpha_of(white), orc.alpha_of(black)
    mask = orc.nft_mask(wa, ba)
    ref = orc.enblend(white, black, mask, seed=3)
    dmask = ctx.nft_mask(_dev(wa), _dev(ba))
    out, oa = ctx.enblend(_dev(white), _dev(black), dmask, seed=3)
    assert np.array_equal(out.cpu().numpy(), ref["out"])
    assert np.array_equal(oa.cpu().numpy(), ref["alpha"])


def test_front_end_generates_seams(orc, tmp_path):
    """enbgpu-enblend --fine-mask --no-optimize on three images: each seam
    from the footprints of the new image and the accumulated result, the
    saved masks equal the oracle's, and the output equals the oracle's chain
    of blends under them."""
    import subprocess
    from enbgpu import _build, synthetic
    bins = {p.name: p for p in _build.build_frontends()}
    h = 120
    # one scene on a 420-wide canvas: image 0 covers columns 0..199 (of the
    # pair's black image, which covers 0..299), images 1 and 2 columns
    # 120..319 and 250..419 (of its white image, which covers 120..419)
    white, black, _ = synthetic.panorama_pair(h, 300, 120, np.uint16, seed=21)
    imgs = []
    for src, lo, hi in ((black, 0, 200), (white, 120, 320), (white, 250, 420)):
        full = np.zeros_like(src)
        full[:, lo:hi] = src[:, lo:hi]
        full[:, lo:hi, 3] = 65535
        imgs.append(full)
    files = []
    for i, x in enumerate(imgs):
        files.append(str(tmp_path / f"in{i}.npy"))
        np.save(files[-1], x)
    out = tmp_path / "out.npy"
    r = subprocess.run([str(bins["enbgpu-enblend"]), "--fine-mask", "--no-optimize",
                        "--save-masks=" + str(tmp_path / "m-%n.npy"), "-o", str(out), *files],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    acc = imgs[0][..., :3].copy()
    acc_alpha = orc.alpha_of(imgs[0])
    for i in (1, 2):
        m = orc.nft_mask(orc.alpha_of(imgs[i]), acc_alpha)
        saved = np.load(tmp_path / f"m-{i}.npy")
        assert np.array_equal(saved, m), i
        ref = orc.enblend(np.ascontiguousarray(imgs[i][..., :3]), acc, m, white_alpha=orc.alpha_of(imgs[i]),
                          black_alpha=acc_alpha, seed=0x5eed)
        acc, acc_alpha = ref["out"], ref["alpha"]
    got = np.load(out)
    assert np.array_equal(got[..., :3], acc)
    assert np.array_equal(got[..., 3], np.where(acc_alpha != 0, 65535, 0).astype(np.uint16))
