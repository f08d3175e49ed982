"""Checkpoint files in the reference's layout (include/Checkpoint.h:26-46).

The fixtures were written by the reference's own Checkpoint::write
(tests/golden/make_golden.py); files written by this library must be
byte-identical to them, and reading them must give back the payload.
Host-only: no GPU needed.
"""
import os

import numpy as np
import pytest

from finitevolume_gb300 import capi, io
from helpers import GOLDEN


def _ref(name):
    return open(os.path.join(GOLDEN, name), "rb").read()


def test_write_is_byte_identical_to_reference(tmp_path):
    pay = np.load(os.path.join(GOLDEN, "ckpt_payloads.npz"))
    p1 = str(tmp_path / "e.bin")
    io.write_checkpoint(p1, "euler", 1234, pay["euler"], build_number=42)
    assert open(p1, "rb").read() == _ref("ckpt_euler_ref.bin")
    p2 = str(tmp_path / "d.bin")
    io.write_checkpoint(p2, "diffusion", 77, pay["diffusion"], build_number=9)
    assert open(p2, "rb").read() == _ref("ckpt_diffusion_ref.bin")


def test_read_reference_checkpoints():
    pay = np.load(os.path.join(GOLDEN, "ckpt_payloads.npz"))
    U, step, build = io.read_checkpoint(os.path.join(GOLDEN, "ckpt_euler_ref.bin"), "euler", 10)
    assert np.array_equal(U, pay["euler"]) and step == 1234 and build == 42
    U2, _, _ = io.read_checkpoint(os.path.join(GOLDEN, "ckpt_euler_ref.bin"), None, 10)  # read_flow_field
    assert np.array_equal(U2, pay["euler"])
    phi, step, build = io.read_checkpoint(os.path.join(GOLDEN, "ckpt_diffusion_ref.bin"), "diffusion", 7)
    assert np.array_equal(phi, pay["diffusion"]) and step == 77 and build == 9


@pytest.mark.parametrize("how", ["equation", "cells", "truncated", "magic", "version"])
def test_read_rejects_mismatches(tmp_path, how):
    src = _ref("ckpt_euler_ref.bin")
    path = str(tmp_path / "bad.bin")
    eq, cells = "euler", 10
    if how == "equation":
        eq = "diffusion"
    elif how == "cells":
        cells = 11
    elif how == "truncated":
        src = src[:-8]
    elif how == "magic":
        src = b"X" + src[1:]
    elif how == "version":
        src = src[:8] + (1).to_bytes(4, "little") + src[12:]
    open(path, "wb").write(src)
    with pytest.raises(capi.FVError) as e:
        io.read_checkpoint(path, eq, cells)
    assert e.value.status == capi.FV_ERR_BAD_ARG


def test_residual_csv(tmp_path):
    p = str(tmp_path / "r.csv")
    w = io.ResidualCSV(p, interval=2)
    for s in range(1, 6):
        w.record(s, [s * 0.1, 2.0, 3.0, 4.0])
    w.close()
    lines = open(p).read().splitlines()
    assert lines[0] == "step,residual_rho,residual_rho_u,residual_rho_v,residual_E"
    assert [l.split(",")[0] for l in lines[1:]] == ["2", "4"]


def test_read_rejects_unknown_equation_tag(tmp_path):
    """An equation tag the format does not define is rejected before any
    payload is read, even when the file carries the same tag."""
    src = bytearray(_ref("ckpt_euler_ref.bin"))
    src[12:16] = (99).to_bytes(4, "little")
    path = str(tmp_path / "tag99.bin")
    open(path, "wb").write(bytes(src))
    out = np.zeros(40)
    st = capi.lib().fv_checkpoint_read(path.encode(), 99, 10, None, None, capi.dptr(out))
    assert st == capi.FV_ERR_BAD_ARG
    assert not out.any()
