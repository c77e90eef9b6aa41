"""Command-line front end: number parsing and argument errors (no GPU needed;
the compute calls are covered by the GPU tests)."""
import pytest

from primecount_gb300.__main__ import parse_number, main
import primecount_gb300 as pcg


def test_parse_number_exact():
    assert parse_number("1e20") == 10 ** 20
    assert parse_number("10^22") == 10 ** 22
    assert parse_number("2^64-1") == 2 ** 64 - 1
    assert parse_number("10**18 + 7") == 10 ** 18 + 7
    assert parse_number("123456789012345678901234567890") == 123456789012345678901234567890
    assert parse_number("3e1") == 30


def test_parse_number_rejects_non_integers():
    for bad in ("1.5", "x", "__import__('os')", "2^1000000"):
        with pytest.raises((ValueError, SyntaxError)):
            parse_number(bad)


def test_argument_errors():
    with pytest.raises(pcg.PrimecountError):
        main(["100", "--phi"])
    with pytest.raises(pcg.PrimecountError):
        main(["100", "200"])
    with pytest.raises(pcg.PrimecountError):
        main([])


@pytest.mark.gpu
def test_cli_results(capsys, golden):
    main(["1e14", "--D"])
    assert capsys.readouterr().out.strip().splitlines()[-1] == "2876480095175"
    main(["1e12", "78498", "--phi"])
    assert capsys.readouterr().out.strip().splitlines()[-1] == "37607833521"
    main(["10^13"])
    assert capsys.readouterr().out.strip().splitlines()[-1] == str(golden["pi_pow10"][str(10 ** 13)])


@pytest.mark.gpu
def test_cli_deleglise_rivat(capsys, golden):
    # -d and the Deleglise-Rivat term options print the reference's values
    row = next(r for r in golden["dr_parts"] if r["x"] == 10 ** 15)
    main(["1e15", "-d"])
    assert capsys.readouterr().out.strip().splitlines()[-1] == str(row["pi"])
    for opt, key in (("--S1", "S1"), ("--S2-trivial", "S2_trivial"), ("--S2-easy", "S2_easy"), ("--P2", "P2")):
        main(["1e15", opt])
        assert capsys.readouterr().out.strip().splitlines()[-1] == str(row[key]), opt


def test_cli_deleglise_rivat_terms_need_large_x():
    with pytest.raises(pcg.PrimecountError):
        main(["1000", "--S2-easy"])
