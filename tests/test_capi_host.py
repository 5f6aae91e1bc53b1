"""C ABI exports and host-side logic (no GPU): the library loads and exports every symbol
declared in include/edgpu.h; operator compilation, restriction masks, codec round trips;
replica sharding over two gloo ranks."""

import os
import re

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from impuritymodel_gb300 import _lib, build

    build()
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "edgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(edgpu_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    from impuritymodel_gb300._lib import SIGNATURES

    assert set(SIGNATURES) == set(names)


def test_abi_version_and_status_strings(lib):
    from impuritymodel_gb300 import _lib as L

    assert lib.edgpu_abi_version() == L.ABI_VERSION == 2
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "edgpu.h")).read()
    assert "#define EDGPU_ABI_VERSION %d" % L.ABI_VERSION in hdr
    assert lib.edgpu_status_string(0) == b"ok"
    assert b"breakdown" in lib.edgpu_status_string(3).lower()


def test_entry_points_reject_bad_arguments_without_a_gpu(lib):
    # argument validation happens before any CUDA call
    from impuritymodel_gb300 import _lib as L

    assert lib.edgpu_apply_columns(0, None, 1, None, None, 0.0, None, 0, 0, None, None, None, None, None, 0, 0, None,
                                   None) == L.EDGPU_ERR_ARG
    assert lib.edgpu_sort_states(9, None, None, 10, None, None, 0, None) == L.EDGPU_ERR_ARG
    assert lib.edgpu_cfrac(None, None, None, 1, 1, None, 1, 0.1, None, None, None, None) == L.EDGPU_ERR_ARG


def test_gemm_tile_width_rule_without_a_gpu(lib):
    """The GEMM's tile width: the widest of 256, 64 and 16 columns dividing N whose grid gives
    four fifths of the SMs a tile, else 16; 0 for shapes the GEMM rejects.  Host-only: without
    a device the library assumes 148 SMs (118 tiles wanted)."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 148
    want = sms * 4 // 5

    def rule(M, N):
        return next((w for w in (256, 64, 16) if N % w == 0 and (M // 128) * (N // w) >= want), 16)

    for M, N in [(128, 256), (4096, 256), (4096, 320), (256, 256), (19456, 256), (65536, 256), (384, 48),
                 (16384, 64), (128, 16)]:
        assert lib.edgpu_gemm_tile_width(M, N) == rule(M, N), (M, N)
    for M, N in [(0, 256), (100, 256), (128, 8), (128, 24), (-128, 64)]:
        assert lib.edgpu_gemm_tile_width(M, N) == 0, (M, N)


def test_noalloc_rejects_bad_arguments_without_a_gpu(lib):
    """edgpu_lanczos_noalloc validates its arguments before any CUDA call: bad precision,
    missing outputs and problems larger than the static scratch array return their codes.
    The pointers below are never dereferenced (host-side stand-ins)."""
    import ctypes as C

    from impuritymodel_gb300 import _lib as L

    fake = C.c_void_p(0x1000)
    csr = L.CSR()
    csr.n, csr.nnz = 1000, 3000
    csr.row_ptr = csr.col = csr.val_r = csr.val_rf = 0x1000
    size = L.noalloc_bytes()
    assert size == lib.edgpu_lanczos_noalloc_bytes() and size > 0

    def call(R=2, K=10, precision=0, alpha=fake, beta=fake, status=fake):
        return lib.edgpu_lanczos_noalloc(C.byref(csr), fake, R, fake, K, precision, alpha, beta, status, None)

    for bad in (-1, 2, 4, 7):
        assert call(precision=bad) == L.EDGPU_ERR_ARG
    assert call(alpha=None) == L.EDGPU_ERR_ARG
    assert call(beta=None) == L.EDGPU_ERR_ARG
    assert call(status=None) == L.EDGPU_ERR_ARG
    assert call(R=0) == L.EDGPU_ERR_ARG
    for prec in (0, 1, 3):
        big_r = 1
        while lib.edgpu_lanczos_workspace(csr.n, big_r, 10, 0 if prec == 3 else prec) <= size:
            big_r *= 2
        assert call(R=big_r, precision=prec) == L.EDGPU_ERR_WORKSPACE
    lib.edgpu_lanczos_noalloc_forget()  # no device state is touched


def test_operator_compilation():
    from impuritymodel_gb300.engine import DeviceOp

    op = {((3, "c"), (3, "a")): 1.5, ((0, "c"), (70, "a")): 0.5 + 0.25j,
          ((1, "c"), (2, "c"), (2, "a"), (1, "a")): -2.0, ((1, "c"), (2, "c"), (4, "a"), (5, "a")): 0.1}
    d = DeviceOp(op, torch.device("cpu"))
    ops = d.ops.numpy().view(np.uint64)
    flags = d.flags.numpy().view(np.uint32)
    assert [int(f) & 1 for f in flags] == [1, 0, 1, 0]
    assert [(int(f) >> 8) & 7 for f in flags] == [2, 2, 4, 4]
    slot = lambda t, k: (int(ops[t]) >> (16 * k)) & 0xFFFF  # noqa: E731
    assert slot(1, 0) == 0x8000 | 0x4000 | 0 and slot(1, 1) == 0x8000 | 70
    assert slot(0, 2) == 0
    assert not d.is_real
    assert np.allclose(d.coeff.numpy()[1], [0.5, 0.25])
    with pytest.raises(ValueError):
        DeviceOp({((0, "x"),): 1.0}, torch.device("cpu"))


def test_restriction_masks():
    from impuritymodel_gb300.engine import make_restrictions

    r = make_restrictions({frozenset([0, 63, 64, 100]): (1, 3)}, 128)
    assert r.n == 1 and r.lo[0] == 1 and r.hi[0] == 3
    assert r.mask[0][0] == (1 << 63) | 1
    assert r.mask[0][1] == (1 << 63) | (1 << (63 - 36))


def test_codec_round_trip():
    from impuritymodel_gb300 import codec

    rng = np.random.default_rng(0)
    for n in (7, 26, 64, 66, 316):
        states = [codec.tuple_to_bytes(tuple(sorted(rng.choice(n, n // 3, replace=False))), n) for _ in range(50)]
        w = codec.bytes_to_words(states, n)
        assert codec.words_to_bytes(w, n) == states
        # lexicographic word order == bytes order
        order = np.lexsort([w[:, q] for q in range(w.shape[1] - 1, -1, -1)])
        assert [states[i] for i in order] == sorted(states)


def test_job_tasks_partition():
    from impuritymodel_gb300.finite import get_job_tasks

    for ranks in (1, 2, 3, 7):
        got = sorted(t for r in range(ranks) for t in get_job_tasks(r, ranks, list(range(50))))
        assert got == list(range(50))


def _replica_worker(rank, world, port, out):
    import torch.distributed as dist

    from impuritymodel_gb300.finite import get_job_tasks

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    mine = list(get_job_tasks(rank, world, list(range(23))))
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t = torch.tensor([0.5 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((sorted(x for g in gathered for x in g), float(t.item())))
    dist.destroy_process_group()


def test_replicas_over_two_gloo_ranks():
    """Independent units (incoming energies) split over ranks with no data exchange; the
    host gathers them and times are reduced with MAX, as bench.py does for N > 1."""
    import socket

    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    units, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert units == list(range(23))
    assert tmax == 1.5
