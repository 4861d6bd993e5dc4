"""Byte-parallel conversion of short rating-text tokens (csrc/text_token.h), on the host:
against strtol/strtof on every token of up to 5 characters over digits, '.', signs, 'e',
control and high bytes, on random longer tokens and on every decimal point position of the
values below 10^6; the space mask against the byte-wise test."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_text_token_matches_strtol_strtof(tmp_path):
    exe = tmp_path / "text_token_check"
    src = os.path.join(HERE, "native", "text_token_check.cpp")
    cc = subprocess.run(["g++", "-O2", "-std=c++17", "-o", str(exe), src], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr + res.stdout
    assert " bad 0" in res.stdout
