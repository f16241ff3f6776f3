"""Host document readers on damaged input: seeded byte mutations and
truncations of the test documents must come back as a status (or a valid
scene), never a crash; deep nesting is refused."""
import numpy as np
import pytest

import spr
from test_rvg import DOC as RVG
from test_svg import DOC as SVG


def mutations(doc, seed, n):
    rng = np.random.default_rng(seed)
    b = bytearray(doc.encode())
    alphabet = b" <>/=\"',.-+eEMLHVCSQAZmlhvcsqaz0123456789()#;:&x\n\t"
    for _ in range(n):
        m = bytearray(b)
        for _ in range(int(rng.integers(1, 6))):
            i = int(rng.integers(0, len(m)))
            op = int(rng.integers(0, 3))
            if op == 0:
                m[i] = alphabet[int(rng.integers(0, len(alphabet)))]
            elif op == 1:
                del m[i]
            else:
                m.insert(i, alphabet[int(rng.integers(0, len(alphabet)))])
        if rng.random() < 0.2:
            m = m[:int(rng.integers(0, len(m)))]
        yield bytes(m)


@pytest.mark.parametrize("kind", ["svg", "rvg"])
def test_mutated_documents(kind):
    doc, parse = (SVG, spr.Scene.parse_svg) if kind == "svg" else (RVG, spr.Scene.parse_rvg)
    ok = 0
    for text in mutations(doc, 17 if kind == "svg" else 18, 400):
        try:
            sc, _ = parse(text)
        except spr.SprError as e:
            assert e.status in (spr.ERR_INVALID_SCENE, spr.ERR_UNSUPPORTED, spr.ERR_INVALID_ARG)
            continue
        ok += 1
        if sc.n_paths:
            assert spr.lib().spr_validate_scene(sc.view()) == spr.OK
            assert np.all(np.isfinite(sc.vertex)) or kind == "rvg"
    assert ok > 0


def test_deep_nesting_is_refused():
    doc = '<svg viewBox="0 0 9 9">' + "<g>" * 300 + '<path d="M0 0 L1 1"/>' + "</g>" * 300 + "</svg>"
    with pytest.raises(spr.SprError) as e:
        spr.Scene.parse_svg(doc)
    assert e.value.status == spr.ERR_INVALID_SCENE
    doc = '<svg viewBox="0 0 9 9">' + "<g>" * 100 + '<path d="M0 0 L1 0 L0 1 z"/>' + "</g>" * 100 + "</svg>"
    sc, _ = spr.Scene.parse_svg(doc)
    assert sc.n_paths == 1


@pytest.mark.parametrize("suffix", ["vgb", "vgt"])
def test_mutated_scene_files(tmp_path, suffix):
    sc, info = spr.Scene.parse_rvg(RVG)
    f = tmp_path / f"doc.{suffix}"
    sc.save_vg(f, info["width"], info["height"])
    data = f.read_bytes()
    rng = np.random.default_rng(23)
    ok = 0
    for _ in range(300):
        m = bytearray(data)
        for _ in range(int(rng.integers(1, 8))):
            i = int(rng.integers(0, len(m)))
            m[i] = int(rng.integers(0, 256)) if suffix == "vgb" else b"0123456789 -.e\n"[int(rng.integers(0, 15))]
        if rng.random() < 0.3:
            m = m[:int(rng.integers(0, len(m)))]
        f.write_bytes(bytes(m))
        try:
            back, _ = spr.Scene.load_vg(f)
        except spr.SprError as e:
            assert e.status in (spr.ERR_INVALID_SCENE, spr.ERR_UNSUPPORTED, spr.ERR_INVALID_ARG,
                                spr.ERR_OUT_OF_MEMORY)
            continue
        ok += 1
        assert spr.lib().spr_validate_scene(back.view()) == spr.OK
    assert ok > 0


def test_scene_file_paths_sharing_one_contour(tmp_path):
    """A small .vgt whose 4,000 paths all name the same 4,000-curve contour:
    the flattening would need 16 M curves, far more than the file's 8,000
    vertices allow, so it must be refused at once (no runaway allocation)."""
    import time

    n_paths, n_curves = 4000, 4000
    out = ["0,0,64,64", f"{n_paths},1,{n_curves},{2 * n_curves},0,0"]
    out += ["0,1,\x00,\x00,4278190335,0"] * n_paths  # contour 0, solid colour, nonzero
    out += [f"0,{n_curves}"]
    out += [f"{2 * i},\x02,-1" for i in range(n_curves)]
    out += [f"{i % 64}.0,{(i * 7) % 64}.0" for i in range(2 * n_curves)]
    f = tmp_path / "shared.vgt"
    f.write_bytes(("\n".join(out) + "\n").encode("latin-1"))
    t0 = time.perf_counter()
    with pytest.raises(spr.SprError) as e:
        spr.Scene.load_vg(f)
    assert e.value.status == spr.ERR_INVALID_SCENE
    assert time.perf_counter() - t0 < 2.0
