"""The block partition of the neighbour-flag FP32 sweep kernel, checked on
the CPU.

The kernel (`sweeps32_local` in ttcode_gb300/csrc/ttfld_mixed.cu) gives
block b of nb the items [n b / nb, n (b + 1) / nb) of one colour, item t
being the vector of four colour slots (k, j, h) with t = (k NY + j) NV + h,
and before each half-sweep waits only for the blocks that own items within
one theta plane (NY NV items) of its own.  That is safe only if every value
of the other colour an item reads (the same row one vector to either side,
the phi rows j - 1 and j + 1 with the periodic wrap, the theta planes
k - 1 and k + 1) belongs to a block in that span; and the relation has to be
symmetric, so that no block overwrites a colour a neighbour is still
reading.  These tests restate the kernel's integer arithmetic and check
both properties for every item of several grids, the ones the GPU tests
use included.
"""
import numpy as np
import pytest


def nv_of(nx):
    """Vectors of four slots per colour row: ceil(ceil(NX / 2) / 4)."""
    nxh = (nx + 1) // 2
    return ((nxh + 3) // 4 * 4) // 4


def owner(t, n, nb):
    """owner_block: the b with n b / nb <= t < n (b + 1) / nb (integer
    division, as in the kernel)."""
    t = np.asarray(t, dtype=np.int64)
    b = t * nb // n
    b = np.where((b + 1 < nb) & (n * (b + 1) // nb <= t), b + 1, b)
    b = np.where((b > 0) & (n * b // nb > t), b - 1, b)
    return b


def span(n, nb, ny, nv):
    """lo, hi of every block: the owners of the items one plane before its
    first item and one plane after its last."""
    b = np.arange(nb, dtype=np.int64)
    t0, t1 = n * b // nb, n * (b + 1) // nb
    reach = ny * nv
    lo = owner(np.maximum(t0 - reach, 0), n, nb)
    hi = owner(np.minimum(t1 - 1 + reach, n - 1), n, nb)
    return lo, hi


def grid_blocks(n, threads=768, sms=152):
    """The kernel's grid: one 768-thread block per SM, at most one block per
    768 items."""
    return int(min(sms, -(-n // threads)))


CASES = [(16, 24, 12), (40, 64, 32), (60, 96, 40), (60, 2048, 6), (100, 128, 64), (100, 256, 128),
         (160, 256, 128), (61, 50, 9)]


@pytest.mark.parametrize("dims", CASES)
def test_owner_matches_the_partition(dims):
    nx, ny, nz = dims
    nv = nv_of(nx)
    n = ny * nz * nv
    nb = grid_blocks(n)
    t = np.arange(n, dtype=np.int64)
    b = owner(t, n, nb)
    b_ref = np.searchsorted(n * np.arange(1, nb + 1, dtype=np.int64) // nb, t, side="right")
    assert np.array_equal(b, b_ref)
    assert np.all(np.bincount(b, minlength=nb) > 0)  # no block without items


@pytest.mark.parametrize("poles", [False, True])
@pytest.mark.parametrize("dims", CASES)
def test_every_read_is_inside_the_span(dims, poles):
    nx, ny, nz = dims
    nv = nv_of(nx)
    n = ny * nz * nv
    nb = grid_blocks(n)
    lo, hi = span(n, nb, ny, nv)
    t = np.arange(n, dtype=np.int64)
    h = t % nv
    j = (t // nv) % ny
    k = t // (nv * ny)
    reads = []
    for dh in (-1, 1):  # the r neighbours across a vector's ends
        ok = (h + dh >= 0) & (h + dh < nv)
        reads.append((ok, t + dh))
    for dj in (-1, 1):  # phi rows, periodic
        jj = (j + dj) % ny
        reads.append((np.ones(n, bool), (k * ny + jj) * nv + h))
    for dk in (-1, 1):  # theta planes; with poles the edge rows read themselves
        kk = k + dk
        ok = (kk >= 0) & (kk < nz)
        if poles:
            ok &= ~(((k == 0) & (dk < 0)) | ((k == nz - 2) & (dk > 0)))
        reads.append((ok, (kk * ny + j) * nv + h))
    bt = owner(t, n, nb)
    for ok, u in reads:
        bu = owner(np.where(ok, u, t), n, nb)
        assert np.all((bu >= lo[bt]) & (bu <= hi[bt])), dims


@pytest.mark.parametrize("dims", CASES)
def test_the_waits_are_symmetric(dims):
    """b waits on c exactly when c waits on b: neighbours stay within one
    half-sweep of each other."""
    nx, ny, nz = dims
    nv = nv_of(nx)
    n = ny * nz * nv
    nb = grid_blocks(n)
    lo, hi = span(n, nb, ny, nv)
    b = np.arange(nb)
    waits = (b[None, :] >= lo[:, None]) & (b[None, :] <= hi[:, None])
    assert np.array_equal(waits, waits.T)


def test_the_gpu_test_grids_cover_one_to_44_neighbours():
    """The grids of the GPU parity test of the flag form: a block waits on
    one to four others on two of them and on up to 44 (more than one flag
    per lane of the polling warp) on the third."""
    widest = {}
    for dims in [(60, 96, 40), (60, 2048, 6), (100, 256, 128)]:
        nx, ny, nz = dims
        nv = nv_of(nx)
        n = ny * nz * nv
        lo, hi = span(n, grid_blocks(n), ny, nv)
        widest[dims] = int(np.max(hi - lo))
    assert widest[(60, 96, 40)] <= 2 and widest[(100, 256, 128)] <= 4
    assert widest[(60, 2048, 6)] == 44
