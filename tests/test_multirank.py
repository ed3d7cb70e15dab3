"""Depth-sharded projection merged across 2 gloo ranks on CPU: the merged
(min, argmin) equals the single-rank oracle result; a rank that fails is seen
by the other on the host, with no collective left waiting."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

LAM, DX = 0.6328, 10.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case():
    from oracle import ref_semantics as ref
    rng = np.random.default_rng(4)
    n, S = 32, 11
    holo = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    return ref.gabor_wavefront(holo), ref.transfer(-1000.0, n, LAM, d), ref.transfer(-200.0, n, LAM, d), S


def _partial(wf, hf, hdz, k0, k1):
    """Oracle min/argmin over slices [k0, k1) of the cumulative slice sequence."""
    from oracle import ref_semantics as ref
    proj = arg = None
    for k, x in enumerate(ref.iter_slices(wf, hf, hdz, k1)):
        if k < k0:
            continue
        inten = ref._intensity(ref._ifft2(ref.ifftshift(x)))
        if proj is None:
            proj, arg = inten, np.full(inten.shape, k, np.int32)
        else:
            better = inten < proj
            arg[better] = k
            proj = np.minimum(proj, inten)
    return proj, arg


def _worker(rank, world, port, q, fail_rank):
    import __graft_entry__ as g
    g.load_package()
    from ph_gb300 import parallel
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wf, hf, hdz, S = _case()
        k0, k1 = parallel.shard_range(S, rank, world)
        store = dist.distributed_c10d._get_default_store()
        if rank == fail_rank:
            store.set(f"failed{rank}", "1")        # announce on the host, then leave between steps
            q.put((rank, "left"))
            return
        if fail_rank >= 0:
            store.wait([f"failed{fail_rank}"])
            q.put((rank, "saw failure"))
            return
        if k1 > k0:
            p, a = _partial(wf, hf, hdz, k0, k1)
            packed = parallel.pack(torch.from_numpy(p), torch.from_numpy(a))
        else:
            packed = parallel.empty_packed((wf.shape[0], wf.shape[1]))
        parallel.merge(packed)
        p, a = parallel.unpack(packed)
        q.put((rank, (p.numpy(), a.numpy())))
    finally:
        dist.destroy_process_group()


def _run(world, fail_rank=-1):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q, fail_rank)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def test_shard_range_covers(ph):
    from ph_gb300 import parallel
    for S in (1, 2, 7, 512):
        for world in (1, 2, 3, 8):
            rs = [parallel.shard_range(S, r, world) for r in range(world)]
            assert sum(k1 - k0 for k0, k1 in rs) == S and rs[0][0] == 0 and rs[-1][1] == S


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_projection_matches_single_rank(ph, world):
    from oracle import ref_semantics as ref
    from ph_gb300 import parallel
    ranges = [parallel.shard_range(11, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == 11
    assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
    out = _run(world)
    wf, hf, hdz, S = _case()
    p_ref, a_ref = ref.reconst_xyprojection(wf, hf, hdz, S, with_argmin=True)
    for r in range(world):
        p, a = out[r]
        assert np.array_equal(p, p_ref)
        assert np.array_equal(a, a_ref)


def test_failed_rank_is_seen_on_host(ph):
    out = _run(2, fail_rank=1)
    assert out[1] == "left" and out[0] == "saw failure"


def test_pack_orders_like_values(ph):
    from ph_gb300 import parallel
    v = torch.tensor([0.0, 1e-30, 0.5, 0.5, 2.0, float("inf")], dtype=torch.float32)
    k = torch.tensor([9, 3, 7, 2, 0, 1], dtype=torch.int32)
    packed = parallel.pack(v, k)
    order = torch.argsort(packed)
    assert order.tolist() == [0, 1, 3, 2, 4, 5]
    p, a = parallel.unpack(packed)
    assert torch.equal(p, v) and torch.equal(a, k)


def test_packed_identity_matches_library_header():
    """The merge identity the gloo ranks use is the library's PH_PACKED_EMPTY, so
    shards produced by ph_reconst_xyproj_range merge with these words as is."""
    import re
    import __graft_entry__ as g
    g.load_package()
    from ph_gb300 import _lib, parallel
    hdr = (g.ROOT / "include" / "phgb300.h").read_text()
    m = re.search(r"#define PH_PACKED_EMPTY (0x[0-9a-fA-F]+)LL", hdr)
    assert m is not None
    assert int(m.group(1), 16) == _lib.PH_PACKED_EMPTY == parallel.PACKED_EMPTY == np.iinfo(np.int64).max
    # every packed word of a non-negative float (finite, inf or NaN) orders below it, signed and unsigned
    for f in (0.0, 1e-30, 1.0, 3.4e38, float("inf"), float("nan")):
        w = parallel.pack(torch.tensor([f], dtype=torch.float32), torch.tensor([0x7FFFFFFF], dtype=torch.int32))
        assert int(w[0]) < parallel.PACKED_EMPTY
