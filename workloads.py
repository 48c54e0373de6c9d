"""Seeded synthetic workloads of the five benchmark configurations.

All generators run on the GPU with torch (plumbing only) and return device
tensors of raw record bytes plus the numpy dtype describing them.  No public
dataset is involved; shapes, sizes and value distributions follow the
configuration descriptions:

  1   1e6 x 12 B [('key','u8'),('value','f4')], uniform keys, value = index
  2a  1e9 x 16 B [('key','u8'),('val','i8')], uniform uint64 keys
  2b  same, keys = arange with 1 % of positions swapped at random
  2c  same, keys = Zipf(s=1.2) ranks over 1e6 distinct values, each rank
      mapped to a seeded random uint64
  3   4096 arrays, sizes round(LogNormal(ln 5e4, 1.5)) clipped to [1, 5e6],
      8 B [('key','i4'),('payload','u4')], keys uniform over int32 with 10 %
      forced to INT32_MIN + [0, 1000)
  4   5e8 x 40 B [('pos',(f4,3)),('vel',(f4,3)),('id','u8'),('key','u8')]:
      positions from 2000 isotropic Gaussians (sigma 0.5-5, log-uniform
      masses as weights) plus 20 % uniform in a periodic 1000^3 box, key =
      21-bit-per-axis Morton code of the position
  5   two snapshots of 2.56e8 x 16 B [('id','i8'),('mass','f4'),('halo','i4')],
      unique ids in [-2^40, 2^40); the second is the first reshuffled with
      2 % dropped and 2 % new ids
"""
import numpy

DT2 = numpy.dtype([('key', 'u8'), ('val', 'i8')])
DT1 = numpy.dtype([('key', 'u8'), ('value', 'f4')])
DT3 = numpy.dtype([('key', 'i4'), ('payload', 'u4')])
DT4 = numpy.dtype([('pos', 'f4', (3,)), ('vel', 'f4', (3,)), ('id', 'u8'), ('key', 'u8')])
DT5 = numpy.dtype([('id', 'i8'), ('mass', 'f4'), ('halo', 'i4')])


def _gen(torch, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return g


def keys_2(torch, n, dist, seed=1234):
    """int64 tensor of uint64 key bits for configuration 2a / 2b / 2c."""
    g = _gen(torch, seed)
    if dist in ("uniform", "2a"):
        return torch.randint(-2**63, 2**63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g)
    if dist in ("sorted1pct", "2b"):
        k = torch.arange(n, dtype=torch.int64, device="cuda")
        m = n // 100
        i = torch.randint(0, n, (m,), device="cuda", generator=g)
        j = torch.randint(0, n, (m,), device="cuda", generator=g)
        ki, kj = k[i].clone(), k[j].clone()
        k[i] = kj
        k[j] = ki
        return k
    if dist in ("zipf", "2c"):
        ranks = torch.arange(1, 10**6 + 1, dtype=torch.float64, device="cuda")
        cdf = torch.cumsum(ranks ** -1.2, 0)
        cdf /= cdf[-1].clone()
        vals = torch.randint(-2**63, 2**63 - 1, (10**6,), dtype=torch.int64, device="cuda", generator=g)
        out = torch.empty(n, dtype=torch.int64, device="cuda")
        step = 1 << 26
        for s in range(0, n, step):
            e = min(n, s + step)
            u = torch.rand(e - s, dtype=torch.float64, device="cuda", generator=g)
            out[s:e] = vals[torch.searchsorted(cdf, u).clamp_(max=10**6 - 1)]
        return out
    raise ValueError(dist)


def records_2(torch, n, dist, seed=1234):
    rec = torch.empty((n, 2), dtype=torch.int64, device="cuda")
    rec[:, 0] = keys_2(torch, n, dist, seed)
    rec[:, 1] = torch.arange(n, device="cuda")
    return rec.view(torch.uint8).view(-1), DT2


def zipf_cdf_int(nv, bits=40):
    """Cumulative integer weights of Zipf(s=1.2) over ranks 1..nv:
    w_r = floor(2^bits * r^-1.2), computed exactly (the float estimate is
    corrected by integer comparisons of w^5 r^6 against 2^(5 bits)), so the
    table is the same on every machine -- no libm pow in the result."""
    r = numpy.arange(1, nv + 1, dtype=numpy.float64)
    w = numpy.floor(numpy.exp2(bits) * r ** -1.2).astype(numpy.int64)
    top = 1 << (5 * bits)
    out = numpy.empty(nv, dtype=numpy.int64)
    for i in range(nv):
        ri6 = (i + 1) ** 6
        x = int(w[i])
        while (x + 1) ** 5 * ri6 <= top:
            x += 1
        while x ** 5 * ri6 > top:
            x -= 1
        out[i] = x
    return numpy.cumsum(out)


def records_2_host(n, dist, seed=2):
    """Configuration 2a / 2b / 2c keys as a numpy record array (PCG64
    seeded, val = index): the host-side twin of keys_2, reproducible
    without a GPU, so that the reference's CPU build can sort the very
    same input."""
    rng = numpy.random.Generator(numpy.random.PCG64(seed))
    a = numpy.empty(n, DT2)
    if dist in ("uniform", "2a"):
        a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    elif dist in ("sorted1pct", "2b"):
        k = numpy.arange(n, dtype=numpy.uint64)
        m = n // 100
        i = rng.integers(0, n, m)
        j = rng.integers(0, n, m)
        ki, kj = k[i].copy(), k[j].copy()
        k[i] = kj
        k[j] = ki
        a['key'] = k
    elif dist in ("zipf", "2c"):
        nv = 10**6
        cdf = zipf_cdf_int(nv)
        vals = rng.integers(0, 2**64, nv, dtype=numpy.uint64, endpoint=False)
        u = rng.integers(0, int(cdf[-1]), n, dtype=numpy.int64)
        a['key'] = vals[numpy.searchsorted(cdf, u, side='right')]
    else:
        raise ValueError(dist)
    a['val'] = numpy.arange(n)
    return a


def records_1(torch, n=10**6, seed=0):
    rng = numpy.random.Generator(numpy.random.PCG64(seed))
    a = numpy.empty(n, DT1)
    a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    a['value'] = numpy.arange(n, dtype=numpy.float32)
    return a


def segments_3(torch, nseg=4096, seed=3):
    """(record bytes on the device, dtype, segment offsets as numpy uint64)."""
    rng = numpy.random.default_rng(seed)
    sizes = numpy.clip(numpy.rint(rng.lognormal(numpy.log(5e4), 1.5, nseg)), 1, 5e6).astype(numpy.int64)
    offs = numpy.concatenate([[0], numpy.cumsum(sizes)]).astype(numpy.uint64)
    n = int(offs[-1])
    g = _gen(torch, seed)
    key = torch.randint(-2**31, 2**31 - 1, (n,), dtype=torch.int64, device="cuda", generator=g)
    near = torch.rand(n, device="cuda", generator=g) < 0.10
    small = torch.randint(0, 1000, (n,), dtype=torch.int64, device="cuda", generator=g)
    key = torch.where(near, -2**31 + small, key)
    rec = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    rec[:, 0] = key.to(torch.int32)
    rec[:, 1] = torch.arange(n, device="cuda", dtype=torch.int64).to(torch.int32)
    return rec.view(torch.uint8).view(-1), DT3, offs


def _morton21(torch, q):
    """Interleave three 21-bit integer coordinates (int64, n x 3) into a
    63-bit Morton code, x in the lowest bit."""
    def spread(v):
        v = v & 0x1FFFFF
        v = (v | (v << 32)) & 0x1F00000000FFFF
        v = (v | (v << 16)) & 0x1F0000FF0000FF
        v = (v | (v << 8)) & 0x100F00F00F00F00F
        v = (v | (v << 4)) & 0x10C30C30C30C30C3
        v = (v | (v << 2)) & 0x1249249249249249
        return v
    return spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)


def particles_4(torch, n=5 * 10**8, seed=4, box=1000.0):
    g = _gen(torch, seed)
    rng = numpy.random.default_rng(seed)
    nc = 2000
    centers = torch.from_numpy(rng.uniform(0, box, (nc, 3)).astype(numpy.float32)).cuda()
    sigma = torch.from_numpy(numpy.exp(rng.uniform(numpy.log(0.5), numpy.log(5.0), nc)).astype(numpy.float32)).cuda()
    mass = numpy.exp(rng.uniform(0, numpy.log(1e3), nc))
    cdf = torch.from_numpy(numpy.cumsum(mass / mass.sum())).cuda()
    rec = torch.empty((n, 10), dtype=torch.int32, device="cuda")
    step = 1 << 25
    for s in range(0, n, step):
        e = min(n, s + step)
        m = e - s
        c = torch.searchsorted(cdf, torch.rand(m, dtype=torch.float64, device="cuda", generator=g)).clamp_(max=nc - 1)
        pos = centers[c] + sigma[c, None] * torch.randn(m, 3, device="cuda", generator=g)
        bg = torch.rand(m, device="cuda", generator=g) < 0.2
        pos = torch.where(bg[:, None], torch.rand(m, 3, device="cuda", generator=g) * box, pos)
        pos = torch.remainder(pos, box)
        vel = torch.randn(m, 3, device="cuda", generator=g)
        q = (pos / box * (1 << 21)).to(torch.int64).clamp_(0, (1 << 21) - 1)
        key = _morton21(torch, q)
        blk = rec[s:e]
        blk[:, 0:3] = pos.view(torch.int32)
        blk[:, 3:6] = vel.view(torch.int32)
        ids = torch.arange(s, e, device="cuda", dtype=torch.int64)
        blk[:, 6:8] = ids.view(torch.int32).view(m, 2)
        blk[:, 8:10] = key.view(torch.int32).view(m, 2)
    return rec.view(torch.uint8).view(-1), DT4


def _id_of(torch, idx):
    """A bijection of [0, 2^41) onto itself (odd multiplier modulo 2^41),
    shifted into [-2^40, 2^40): distinct indices give distinct ids."""
    a = 0x1D872B41D3  # odd
    return ((idx * a + 0x5A5A5A5) & ((1 << 41) - 1)) - (1 << 40)


def snapshots_5(torch, n=256 * 10**6, seed=5):
    """(bytes of A followed by B on the device, dtype, n_a, n_b, expected
    number of common ids)."""
    g = _gen(torch, seed)
    ia = torch.arange(n, device="cuda", dtype=torch.int64)
    ia = ia[torch.randperm(n, device="cuda", generator=g)]
    drop = n // 50
    keep = ia[drop:]                       # 2 % of A's ids dropped
    new = torch.arange(n, n + drop, device="cuda", dtype=torch.int64)  # 2 % new ids
    ib = torch.cat([keep, new])
    ib = ib[torch.randperm(len(ib), device="cuda", generator=g)]
    recs = torch.zeros((len(ia) + len(ib), 4), dtype=torch.int32, device="cuda")
    ids = torch.cat([_id_of(torch, ia), _id_of(torch, ib)])
    recs[:, 0:2] = ids.view(torch.int32).view(-1, 2)
    recs[:, 2] = torch.rand(len(ids), device="cuda", generator=g).view(torch.int32)
    recs[:, 3] = torch.randint(0, 10**6, (len(ids),), device="cuda", generator=g, dtype=torch.int32)
    return recs.view(torch.uint8).view(-1), DT5, len(ia), len(ib), len(keep)


def device_parity(torch, rec, out, n, key_col=0, ident_col=1, segment_start=None, signed=False):
    """Size-independent parity of a sort of records whose `ident_col` word
    holds the input index (integer tensors of shape (n, words) on the device,
    input `rec` and output `out`):
      key_payload  out[i].key == rec[out[i].ident].key for every i (each
                   output record is the input record it names), and the
                   record stayed in its segment;
      permutation  every input index appears exactly once;
      sorted       keys ascend (within each segment, if segment_start is a
                   bool mask of segment first positions);
      stable       equal keys keep ascending input index.
    Together these pin the unique stable order record for record.  Keys are
    compared as unsigned (signed=False: int64 words flipped into int64
    order) or as signed integers."""
    step = 1 << 27
    ok_kp = ok_sorted = ok_stable = True
    seen = torch.zeros(n, dtype=torch.int32, device=rec.device)
    seg_id = None
    if segment_start is not None:
        seg_id = torch.cumsum(segment_start.to(torch.int32), 0, dtype=torch.int32)
    for s in range(0, n, step):
        e = min(n, s + step)
        ident = out[s:e, ident_col].long()
        if bool(((ident < 0) | (ident >= n)).any().item()):
            return {"key_payload": False, "permutation": False, "sorted": False, "stable": False}
        ok_kp &= bool(torch.equal(out[s:e, key_col], rec[ident, key_col]))
        if seg_id is not None:
            ok_kp &= bool(torch.equal(seg_id[ident], seg_id[s:e]))
        seen.index_add_(0, ident, torch.ones_like(ident, dtype=torch.int32))
        e1 = min(n, e + 1)
        k = out[s:e1, key_col]
        if not signed:
            k = k ^ (-2**63)
        up = k[1:] >= k[:-1]
        tie_ok = (k[1:] != k[:-1]) | (out[s + 1:e1, ident_col] > out[s:e1 - 1, ident_col])
        if segment_start is not None:
            first = segment_start[s + 1:e1]
            up |= first
            tie_ok |= first
        ok_sorted &= bool(up.all().item())
        ok_stable &= bool(tie_ok.all().item())
    ok_perm = bool((seen == 1).all().item())
    return {"key_payload": ok_kp, "permutation": ok_perm, "sorted": ok_sorted, "stable": ok_stable}
