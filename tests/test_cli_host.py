"""Host-side parts of the benchmark CLI (gbsort.cli) that need no GPU: the
reference's C type names, its value types and input modes, the statistics
it prints, the validation size limit, and a clean exit without a device."""

import pytest

from gbsort import cli


def test_type_names_cover_every_key_type(gb):
    assert set(cli.TYPE_NAMES.values()) == set(gb.KEY_TYPES)
    for c_name, short in cli.TYPE_NAMES.items():
        assert cli.key_type(c_name) == short
        assert cli.key_type(short) == short
    # the reference's validation order names every type once
    assert sorted(cli.key_type(t) for t in cli.VALIDATION_TYPES) == sorted(gb.KEY_TYPES)
    with pytest.raises(SystemExit):
        cli.key_type("uint24_t")


def test_value_types_and_modes(gb):
    assert cli.VALUE_TYPES == {"none": 0, "uint32_t": 4, "uint8_t": 1, "uint16_t": 2, "uint64_t": 8,
                               "unsigned __int128": 16}
    assert set(cli.MODES) == {"random", "byte_skip", "asc"}


def test_stats():
    st = cli.stats([1.0, 2.0, 3.0, 4.0, 100.0])
    assert st["avg"] == pytest.approx(22.0)
    assert st["p50"] == 3.0 and st["p99"] == 100.0
    assert st["std_us"] > 0
    assert cli.stats([5.0])["std_us"] == 0.0


def test_max_array_bits():
    gib = 1 << 30
    assert cli.max_array_bits(280 * gib, 8) == 31  # 70 GiB / 24 B
    assert cli.max_array_bits(1 << 12, 16) == 10  # never below 2^10
    for b in (4, 8, 16, 32):
        bits = cli.max_array_bits(280 * gib, b)
        assert (1 << bits) * 3 * b <= 280 * gib // 4 < (1 << (bits + 1)) * 3 * b


def test_main_without_device(capsys):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    assert cli.main(["--n", "1024"]) == 2
    assert "no CUDA device" in capsys.readouterr().err
    with pytest.raises(SystemExit):
        cli.main(["--values", "float"])  # not a value type of the reference
