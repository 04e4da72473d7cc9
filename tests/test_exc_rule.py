"""Bit-exact parity of the excitation rule (partner determinant + fermionic sign)
against the reference's applyExcToBasisState_ (fusedevolve.cpp:27-145).

The golden tables were dumped by the reference itself (tests/golden/make_golden.py):
f90 and syn6 over every bitstring of their full spaces; pairs12 over every
determinant of the 12-orbital 6a+6b sector for all 165 operators of the 3-layer TUPS
circuit, as SHA-256 digests of the partner and sign arrays plus raw samples.
The host rule (the one the orbit tables are built with) is checked on CPU; the device
rule (the one the pass kernels evaluate), over the engine's own sector basis, on the GPU.
"""
import hashlib

import numpy as np
import pytest

import ansatzevolve_gb300 as ae


def _u32p(a):
    import ctypes
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _i8p(a):
    import ctypes
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))


def sector_list(N, na, nb):
    pc = np.array([bin(v).count("1") for v in range(1 << N)])
    a = np.flatnonzero(pc == na).astype(np.uint32)
    b = np.flatnonzero(pc == nb).astype(np.uint32)
    return ((a[:, None] << np.uint32(N)) | b[None, :]).ravel()


def host_rule(ops0, states):
    ops0 = np.ascontiguousarray(ops0, dtype=np.int32).reshape(-1, 4)
    states = np.ascontiguousarray(states, dtype=np.uint32)
    n = len(states)
    partner = np.zeros(len(ops0) * n, dtype=np.uint32)
    sign = np.zeros(len(ops0) * n, dtype=np.int8)
    rc = ae.lib().aegpu_host_exc_rule(len(ops0), ae.iptr(ops0.ravel()), _u32p(states), n, _u32p(partner), _i8p(sign))
    assert rc == 0
    return partner.reshape(len(ops0), n), sign.reshape(len(ops0), n)


def check_digests(fx, partner, sign, ops_slice):
    for k, o in enumerate(ops_slice):
        assert hashlib.sha256(partner[k].astype("<u4").tobytes()).hexdigest() == str(fx["partner_sha256"][o]), o
        assert hashlib.sha256(sign[k].tobytes()).hexdigest() == str(fx["sign_sha256"][o]), o
        pick = fx["sample_rank"]
        np.testing.assert_array_equal(partner[k][pick], fx["sample_partner"][o])
        np.testing.assert_array_equal(sign[k][pick], fx["sample_sign"][o])


@pytest.mark.parametrize("name", ["f90", "syn6"])
def test_host_rule_matches_reference_full_tables(golden, name):
    fx = golden(name)
    ops0 = np.asarray(fx["ops_1b"]) - 1
    nq = int(fx["nq"]) if "nq" in fx else 2 * int(fx["N"])
    states = np.arange(1 << nq, dtype=np.uint32)
    partner, sign = host_rule(ops0, states)
    np.testing.assert_array_equal(partner, fx["pair_partner"])
    np.testing.assert_array_equal(sign, fx["pair_sign"])


def test_host_rule_matches_reference_12_orbitals(golden):
    fx = golden("pairs12")
    N, na, nb = int(fx["N"]), int(fx["na"]), int(fx["nb"])
    sect = sector_list(N, na, nb)
    assert hashlib.sha256(sect.astype("<u4").tobytes()).hexdigest() == str(fx["sector_sha256"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    for o0 in range(0, len(ops0), 33):
        part, sg = host_rule(ops0[o0:o0 + 33], sect)
        check_digests(fx, part, sg, range(o0, min(o0 + 33, len(ops0))))
        for k in range(part.shape[0]):
            assert int(np.count_nonzero(part[k] != sect)) == int(fx["active"][o0 + k])


@pytest.mark.gpu
def test_device_rule_matches_reference_12_orbitals(golden):
    """Every operator of the 12-orbital circuit over every determinant of the engine's own
    6a+6b basis (which must equal the reference's ascending sector list), on the GPU."""
    torch = pytest.importorskip("torch")
    fx = golden("pairs12")
    N, na, nb = int(fx["N"]), int(fx["na"]), int(fx["nb"])
    ops0 = (np.asarray(fx["ops_1b"]) - 1).astype(np.int32)
    eng = ae.Engine(2 * N, ae.BASIS_SZ, na + nb, na, nb, ops0)
    sect = eng.states().astype(np.uint32)
    assert hashlib.sha256(sect.astype("<u4").tobytes()).hexdigest() == str(fx["sector_sha256"])
    n = len(sect)
    dev = torch.device("cuda")
    st = torch.from_numpy(sect.view(np.int32)).to(dev)
    step = 33
    part = torch.empty(step * n, dtype=torch.int32, device=dev)
    sg = torch.empty(step * n, dtype=torch.int8, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for o0 in range(0, len(ops0), step):
        blk = np.ascontiguousarray(ops0[o0:o0 + step])
        rc = ae.lib().aegpu_exc_rule_dev(len(blk), ae.iptr(blk.ravel()), st.data_ptr(), n, part.data_ptr(),
                                         sg.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        p = part[:len(blk) * n].cpu().numpy().view(np.uint32).reshape(len(blk), n)
        s = sg[:len(blk) * n].cpu().numpy().reshape(len(blk), n)
        check_digests(fx, p, s, range(o0, o0 + len(blk)))
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["f90", "syn6"])
def test_device_rule_matches_reference_full_tables(golden, name):
    torch = pytest.importorskip("torch")
    fx = golden(name)
    ops0 = np.ascontiguousarray(np.asarray(fx["ops_1b"]) - 1, dtype=np.int32)
    nq = int(fx["nq"]) if "nq" in fx else 2 * int(fx["N"])
    n = 1 << nq
    dev = torch.device("cuda")
    st = torch.arange(n, dtype=torch.int32, device=dev)
    part = torch.empty(len(ops0) * n, dtype=torch.int32, device=dev)
    sg = torch.empty(len(ops0) * n, dtype=torch.int8, device=dev)
    rc = ae.lib().aegpu_exc_rule_dev(len(ops0), ae.iptr(ops0.ravel()), st.data_ptr(), n, part.data_ptr(),
                                     sg.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(part.cpu().numpy().view(np.uint32).reshape(len(ops0), n), fx["pair_partner"])
    np.testing.assert_array_equal(sg.cpu().numpy().reshape(len(ops0), n), fx["pair_sign"])
