"""Grid documents: the reference's text format printed back from a dense grid,
and the binary dense-grid format beside it (host only, no GPU needed)."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_parse.jsonl")
CLI = os.path.join(ROOT, "cuda_a_star_gb300", "_build", "astar_gpu")


def _golden_grids():
    with open(GOLDEN) as f:
        return [d for d in map(json.loads, f) if d["kind"] == "grid_parse"]


@pytest.mark.parametrize("case", range(len(_golden_grids())))
def test_text_round_trip_of_reference_documents(gastar, case):
    d = _golden_grids()[case]
    wts, st, gl = gastar.parse_grid(d["input"])
    text = gastar.format_grid(wts, st, gl)
    w2, s2, g2 = gastar.parse_grid(text)
    assert np.array_equal(wts, w2) and s2 == st and g2 == gl


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_binary_round_trip(gastar, seed):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(1, 300)), int(rng.integers(1, 300))
    wts = gastar.gen_grid(w, h, seed, 0.2)
    st = (int(rng.integers(0, w)), int(rng.integers(0, h)))
    gl = (int(rng.integers(0, w)), int(rng.integers(0, h)))
    blob = gastar.encode_grid_binary(wts, st, gl)
    assert len(blob) == 32 + w * h and blob[:8] == b"GAGRID1\0"
    assert int.from_bytes(blob[8:12], "little") == w and int.from_bytes(blob[12:16], "little") == h
    w2, s2, g2 = gastar.decode_grid_binary(blob)
    assert np.array_equal(wts, w2) and s2 == st and g2 == gl
    # text and binary describe the same grid
    w3, s3, g3 = gastar.parse_grid(gastar.format_grid(wts, st, gl))
    assert np.array_equal(w3, wts) and (s3, g3) == (st, gl)


def test_binary_rejects_malformed(gastar):
    wts = gastar.gen_grid(8, 5, 9, 0.2)
    blob = gastar.encode_grid_binary(wts, (0, 0), (7, 4))
    with pytest.raises(gastar.GastarError):
        gastar.decode_grid_binary(b"NOTAGRID" + blob[8:])
    with pytest.raises(gastar.GastarError):
        gastar.decode_grid_binary(blob[:-1])          # truncated weights
    bad = bytearray(blob)
    bad[16:20] = (8).to_bytes(4, "little")           # start x outside the board
    with pytest.raises(gastar.GastarError):
        gastar.decode_grid_binary(bytes(bad))
    with pytest.raises(gastar.GastarError):
        gastar.encode_grid_binary(wts, (8, 0), (7, 4))


def test_cli_converts_between_formats(gastar, tmp_path):
    assert os.path.exists(CLI)
    wts = gastar.gen_grid(64, 48, 17, 0.25)
    txt = tmp_path / "g.txt"
    txt.write_text(gastar.format_grid(wts, (1, 2), (60, 40)))
    binf, back = tmp_path / "g.bin", tmp_path / "g2.txt"
    p = subprocess.run([CLI, "--version", "pathfinding", "--input-data", str(txt), "--convert",
                        "binary", "--output-data", str(binf)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout
    w2, s2, g2 = gastar.decode_grid_binary(binf.read_bytes())
    assert np.array_equal(w2, wts) and s2 == (1, 2) and g2 == (60, 40)
    p = subprocess.run([CLI, "--version", "pathfinding", "--input-format", "binary", "--input-data",
                        str(binf), "--convert", "text", "--output-data", str(back)],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stdout
    w3, s3, g3 = gastar.parse_grid(back.read_text())
    assert np.array_equal(w3, wts) and (s3, g3) == ((1, 2), (60, 40))
    p = subprocess.run([CLI, "--version", "sliding", "--convert", "binary"], capture_output=True,
                       text=True, input="")
    assert p.returncode == 255
