"""SpMV parity on the GPU: every variant, through the C ABI, against the oracle.

x is random in [-1, 1] (never all ones, unlike main.cpp:27), so layout bugs
that a constant x hides (the reference's coal-x staging) show up. Each y
carries a guard tail that must stay untouched.
"""
import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm
from conftest import golden_cases, load_golden, spmv_tolerance

pytestmark = pytest.mark.gpu

TEMPLATE_BS = {1, 2, 3, 4, 8, 16, 32}
BCSR_VARIANTS = [bm.BCSR_ROW_THREAD, bm.BCSR_ROW_WARP, bm.BCSR_COL_THREAD, bm.BCSR_COL_THREAD_TEMPLATE,
                 bm.BCSR_COL_COAL_X, bm.BCSR_COL_COAL_X_TEMPLATE, bm.BCSR_COL_BY_COL,
                 bm.BCSR_COL_BY_COL_FASTDIV, bm.BCSR_COL_BY_COL_PO2, bm.BCSR_COL_BY_COL_TEMPLATE,
                 bm.BCSR_JIT, bm.CUSPARSE_ROW, bm.CUSPARSE_COL, bm.BCSR_NATIVE]
GUARD = 16


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def expected_support(variant, bs):
    templ = {bm.BCSR_ROW_WARP, bm.BCSR_COL_THREAD_TEMPLATE, bm.BCSR_COL_COAL_X_TEMPLATE,
             bm.BCSR_COL_BY_COL_TEMPLATE, bm.BCSR_JIT}
    if variant in templ and bs not in TEMPLATE_BS:
        return False
    if variant in (bm.BCSR_COL_BY_COL, bm.BCSR_COL_BY_COL_FASTDIV, bm.BCSR_COL_BY_COL_PO2) and bs > 32:
        return False
    if variant == bm.BCSR_COL_BY_COL_PO2 and bs & (bs - 1):
        return False
    if variant in (bm.CUSPARSE_ROW, bm.CUSPARSE_COL) and bs == 1:
        return False
    return True


def ragged_bcsr(nbr, nbc, bs, seed, dtype, max_blocks=12):
    """Random BCSR with empty block rows and 0..max_blocks sorted blocks per row."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(0, max_blocks + 1, nbr)
    counts[rng.random(nbr) < 0.15] = 0
    counts = np.minimum(counts, nbc)
    rp = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    cols = np.concatenate([np.sort(rng.choice(nbc, size=k, replace=False)) for k in counts]
                          or [np.zeros(0)]).astype(np.int32)
    vals = rng.uniform(-1, 1, int(rp[-1]) * bs * bs).astype(dtype)
    return rp, cols, vals


def run_variant(orc, variant, rp, cols, vals, bs, nbc, dtype, seed=0, x_offset=0):
    import torch
    n_out = (rp.size - 1) * bs
    x_np = np.random.default_rng(seed + 100).uniform(-1, 1, nbc * bs + x_offset).astype(dtype)
    vals_in = orc.transpose_blocks(rp, vals, bs) if bm.variant_layout(variant) == 1 else vals
    d_rp, d_c, d_v = dev(rp), dev(cols), dev(vals_in)
    d_xfull = dev(x_np)
    d_x = d_xfull[x_offset:]
    d_y = torch.full((n_out + GUARD,), float("nan"), dtype=d_v.dtype, device="cuda")
    bm.bcsr_spmv(variant, d_rp, d_c, d_v, d_x, d_y, bs, nbc)
    torch.cuda.synchronize()
    y = d_y.cpu().numpy()
    assert np.isnan(y[n_out:]).all(), "write past the end of y"
    x = x_np[x_offset:]
    y_ref = orc.bcsr_spmv(rp, cols, vals, bs, x)
    crp, cc, cv = orc.bcsr_to_csr(rp, cols, vals, bs)
    tol = spmv_tolerance(orc, crp, cc, cv, x, dtype)
    err = np.abs(y[:n_out].astype(np.float64) - y_ref.astype(np.float64))
    assert np.all(err <= tol), (bm.variant_name(variant), float((err - tol).max()))
    if n_out and np.any(y_ref):
        _, flagged = orc.compare_results(y[:n_out].astype(dtype), y_ref)
        assert not flagged


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [1, 2, 3, 4, 5, 8, 16, 32])
@pytest.mark.parametrize("variant", BCSR_VARIANTS)
def test_bcsr_variant_parity_band(lib, orc, cuda, variant, bs, dtype):
    nbr = 300 if bs <= 8 else 90
    rp, c, v = bm.gen_band_bcsr(nbr, 8, 64, bs, seed=bs, dtype=dtype)
    if not expected_support(variant, bs):
        with pytest.raises(bm.BmfpError) as e:
            run_variant(orc, variant, rp, c, v, bs, nbr, dtype)
        assert e.value.status == bm.ERROR_NOT_SUPPORTED
        return
    run_variant(orc, variant, rp, c, v, bs, nbr, dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [1, 2, 3, 4, 8, 16, 32])
@pytest.mark.parametrize("variant", BCSR_VARIANTS)
def test_bcsr_variant_parity_ragged(lib, orc, cuda, variant, bs, dtype):
    if not expected_support(variant, bs):
        pytest.skip("variant not instantiated for this block size")
    rp, c, v = ragged_bcsr(157, 131, bs, seed=bs + 7, dtype=dtype)
    run_variant(orc, variant, rp, c, v, bs, 131, dtype, seed=bs)


@pytest.mark.parametrize("variant", [bm.BCSR_ROW_THREAD, bm.BCSR_COL_THREAD, bm.BCSR_COL_COAL_X, bm.BCSR_NATIVE])
@pytest.mark.parametrize("bs", [33, 40])
def test_bcsr_large_block_sizes(lib, orc, cuda, variant, bs):
    rp, c, v = ragged_bcsr(20, 17, bs, seed=bs, dtype=np.float64, max_blocks=4)
    run_variant(orc, variant, rp, c, v, bs, 17, np.float64)


@pytest.mark.parametrize("name", golden_cases("ndiag_") + ["bridge_f64.npz"])
@pytest.mark.parametrize("variant", [bm.BCSR_NATIVE, bm.BCSR_COL_COAL_X, bm.BCSR_COL_BY_COL, bm.BCSR_ROW_WARP])
def test_bcsr_parity_on_reference_matrices(lib, orc, cuda, name, variant):
    g = load_golden(name)
    bs = int(g["bs"])
    if not expected_support(variant, bs):
        pytest.skip("variant not instantiated for this block size")
    run_variant(orc, variant, g["bcsr_row_ptr"], g["bcsr_cols"], g["bcsr_vals"], bs, int(g["n_block_cols"]),
                g["bcsr_vals"].dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [2, 4, 8, 16, 32])
def test_native_every_lane_count(lib, orc, cuda, bs, dtype):
    import torch
    nbr = 200 if bs <= 8 else 60
    rp, c, v = ragged_bcsr(nbr, nbr, bs, seed=3 * bs, dtype=dtype, max_blocks=20)
    x = np.random.default_rng(1).uniform(-1, 1, nbr * bs).astype(dtype)
    y_ref = orc.bcsr_spmv(rp, c, v, bs, x)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    tol = spmv_tolerance(orc, crp, cc, cv, x, dtype)
    vec = 2 if dtype == np.float64 else 4
    for g in (2, 4, 8, 16, 32, 64):  # 64 = BMFP_LANES_ROW_OWNER (one lane per scalar row)
        if g == 64 and bs < 4:
            continue
        d_y = torch.full((nbr * bs + GUARD,), float("nan"), dtype=torch.float64 if dtype == np.float64 else torch.float32,
                         device="cuda")
        if g != 64 and g * vec < bs:
            with pytest.raises(bm.BmfpError):
                bm.bcsr_spmv_native(dev(rp), dev(c), dev(v), dev(x), d_y, bs, lanes=g)
            continue
        bm.bcsr_spmv_native(dev(rp), dev(c), dev(v), dev(x), d_y, bs, lanes=g)
        y = d_y.cpu().numpy()
        assert np.isnan(y[nbr * bs:]).all()
        assert np.all(np.abs(y[:nbr * bs] - y_ref) <= tol), g


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [1, 2, 4, 8])
def test_native_misaligned_x_falls_back(lib, orc, cuda, bs, dtype):
    rp, c, v = bm.gen_band_bcsr(120, 8, 64, bs, seed=2, dtype=dtype)
    run_variant(orc, bm.BCSR_NATIVE, rp, c, v, bs, 120, dtype, x_offset=1)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("variant", [bm.CSR_SCALAR, bm.CSR_VECTOR, bm.CSR_NATIVE])
@pytest.mark.parametrize("bs", [1, 3, 8])
def test_csr_variant_parity(lib, orc, cuda, variant, bs, dtype):
    import torch
    rp, c, v = ragged_bcsr(150, 140, bs, seed=bs, dtype=dtype)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    n = (rp.size - 1) * bs
    x = np.random.default_rng(4).uniform(-1, 1, 140 * bs).astype(dtype)
    d_y = torch.full((n + GUARD,), float("nan"), dtype=torch.float64 if dtype == np.float64 else torch.float32,
                     device="cuda")
    bm.csr_spmv(variant, dev(crp), dev(cc), dev(cv), dev(x), d_y)
    y = d_y.cpu().numpy()
    assert np.isnan(y[n:]).all()
    y_ref = orc.csr_spmv(crp, cc, cv, x)
    assert np.all(np.abs(y[:n] - y_ref) <= spmv_tolerance(orc, crp, cc, cv, x, dtype))


def test_empty_and_zero_block_matrices(lib, orc, cuda):
    import torch
    # no block rows at all: a valid no-op
    assert lib.bmfp_bcsr_spmv(bm.R64F, bm.BCSR_NATIVE, 0, 0, 2, 0, None, None, None, None, None, None) == 0
    # rows but no blocks: y must be exactly zero
    rp = np.zeros(11, np.int32)
    d_y = torch.full((20,), 5.0, dtype=torch.float64, device="cuda")
    x = torch.ones(20, dtype=torch.float64, device="cuda")
    for variant in (bm.BCSR_NATIVE, bm.BCSR_ROW_THREAD, bm.BCSR_COL_BY_COL):
        d_y.fill_(5.0)
        bm.bcsr_spmv(variant, dev(rp), torch.zeros(1, dtype=torch.int32, device="cuda"),
                     torch.zeros(4, dtype=torch.float64, device="cuda"), x, d_y, 2, 10)
        torch.cuda.synchronize()
        assert (d_y.cpu() == 0).all()


@pytest.mark.parametrize("bs", [2, 4, 8])
def test_matrix_handle_upload_autotune_convert(lib, orc, cuda, bs):
    import torch
    rp, c, v = bm.gen_band_bcsr(2000, 8, 64, bs, seed=5)
    m = bm.Matrix.from_bcsr(rp, c, v, bs)
    x = np.random.default_rng(0).uniform(-1, 1, 2000 * bs)
    d_x = dev(x)
    d_y = torch.empty(2000 * bs, dtype=torch.float64, device="cuda")
    lanes = m.autotune(d_x, d_y)
    assert lanes in (2, 4, 8, 16, 32, 64)
    m.spmv(d_x, d_y)
    y_ref = orc.bcsr_spmv(rp, c, v, bs, x)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    assert np.all(np.abs(d_y.cpu().numpy() - y_ref) <= spmv_tolerance(orc, crp, cc, cv, x, np.float64))
    assert m.bytes_per_spmv() == bm.bcsr_spmv_bytes(np.float64, 2000, 2000, bs, c.size)
    m32 = m.convert(np.float32)
    y32 = torch.empty(2000 * bs, dtype=torch.float32, device="cuda")
    m32.spmv(d_x.float(), y32)
    v32, x32 = v.astype(np.float32), x.astype(np.float32)
    y32_ref = orc.bcsr_spmv(rp, c, v32, bs, x32)
    assert np.all(np.abs(y32.cpu().numpy() - y32_ref) <= spmv_tolerance(orc, crp, cc, cv.astype(np.float32), x32,
                                                                       np.float32))
    m.close(), m32.close()


@pytest.mark.parametrize("bs,dtype", [(1, np.float64), (2, np.float64), (4, np.float64), (8, np.float64),
                                      (2, np.float32), (8, np.float32)])
def test_full_size_band_sweep_parity(lib, orc, cuda, bs, dtype):
    """The block-size sweep workload at its full size (100 000 block rows,
    8 blocks per row, +-64 band) against the oracle, every entry."""
    import torch
    nbr = 100_000
    rp, c, v = bm.gen_band_bcsr(nbr, 8, 64, bs, seed=0, dtype=dtype)
    x = bm.gen_uniform_vector(nbr * bs, 0, 2, dtype)
    m = bm.Matrix.from_bcsr(rp, c, v, bs)
    d_y = torch.empty(nbr * bs, dtype=torch.float64 if dtype == np.float64 else torch.float32, device="cuda")
    m.spmv(dev(x), d_y)
    y = d_y.cpu().numpy()
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    y_ref = orc.csr_spmv(crp, cc, cv, x, threads=8)
    assert np.all(np.abs(y - y_ref) <= spmv_tolerance(orc, crp, cc, cv, x, dtype))
    m.close()


@pytest.mark.parametrize("bs,dtype,pinned", [(1, np.float64, True), (2, np.float64, True), (3, np.float64, False),
                                             (4, np.float64, True), (8, np.float32, True), (32, np.float64, False),
                                             (16, np.float32, False)])
def test_host_buffer_spmv_chunked(lib, orc, cuda, bs, dtype, pinned):
    """bmfp_bcsr_spmv_host: host arrays in, host y out, the upload split into
    block-row chunks with the product of each chunk overlapping the next
    upload. Sizes are picked so that most cases cut the matrix into several
    chunks (8 MB each at least), including ragged rows and empty rows."""
    import torch
    nbr = 60_000 if bs <= 4 else 6_000
    rp, c, v = ragged_bcsr(nbr, nbr, bs, seed=bs, dtype=dtype, max_blocks=16)
    x = np.random.default_rng(bs).uniform(-1, 1, nbr * bs).astype(dtype)
    if pinned:
        pin = [torch.from_numpy(a).pin_memory() for a in (rp, c, v, x)]
        rp, c, v, x = (t.numpy() for t in pin)
    y = bm.bcsr_spmv_host(rp, c, v, x, bs)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    y_ref = orc.csr_spmv(crp, cc, cv, x, threads=8)
    assert np.all(np.abs(y - y_ref) <= spmv_tolerance(orc, crp, cc, cv, x, dtype))
    # repeated calls reuse the pooled device memory and give the same bits
    assert np.array_equal(bm.bcsr_spmv_host(rp, c, v, x, bs).view(np.uint8), y.view(np.uint8))


def test_host_buffer_spmv_edges(lib, orc, cuda):
    # no rows, no blocks (y = 0), and a malformed row_ptr refused before any copy
    assert bm.bcsr_spmv_host(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), 2).size == 0
    y = bm.bcsr_spmv_host(np.zeros(5, np.int32), np.zeros(0, np.int32), np.zeros(0), np.ones(8), 2)
    assert np.array_equal(y, np.zeros(8))
    with pytest.raises(bm.BmfpError) as e:
        bm.bcsr_spmv_host(np.array([0, 2], np.int32), np.zeros(1, np.int32), np.zeros(4), np.ones(2), 2)
    assert e.value.status == bm.ERROR_INVALID_VALUE


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [2, 4, 8, 16, 32])
def test_column_owner_mapping(lib, orc, cuda, bs, dtype):
    """BMFP_LANES_COL_OWNER: the handle keeps a column-major copy of its blocks
    and one lane per scalar row walks its columns; same parity bar as every
    other mapping, on ragged rows with empty rows. Switching back releases
    the copy and gives the row-major kernel's result again."""
    import torch
    nbr = 3000 if bs <= 8 else 600
    rp, c, v = ragged_bcsr(nbr, nbr, bs, seed=bs + 50, dtype=dtype)
    x = np.random.default_rng(bs).uniform(-1, 1, nbr * bs).astype(dtype)
    m = bm.Matrix.from_bcsr(rp, c, v, bs)
    dx = dev(x)
    dy = torch.empty_like(dx)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    y_ref = orc.csr_spmv(crp, cc, cv, x, threads=8)
    tol = spmv_tolerance(orc, crp, cc, cv, x, dtype)
    m.set_lanes(bm.LANES_COL_OWNER)
    m.spmv(dx, dy)
    assert np.all(np.abs(dy.cpu().numpy() - y_ref) <= tol)
    m.set_lanes(0)
    m.spmv(dx, dy)
    assert np.all(np.abs(dy.cpu().numpy() - y_ref) <= tol)
    lanes = m.autotune(dx, dy)  # may pick the column owner again
    m.spmv(dx, dy)
    assert np.all(np.abs(dy.cpu().numpy() - y_ref) <= tol), lanes
    m.close()


def test_column_owner_rejected_where_it_does_not_apply(lib, cuda):
    rp, c, v = ragged_bcsr(100, 100, 3, seed=1, dtype=np.float64)
    m = bm.Matrix.from_bcsr(rp, c, v, 3)
    with pytest.raises(bm.BmfpError):
        m.set_lanes(bm.LANES_COL_OWNER)
    m.close()


def test_lane_choices_the_matrix_cannot_run_are_refused(lib, cuda):
    rp, c, v = ragged_bcsr(100, 100, 2, seed=3, dtype=np.float64)
    m = bm.Matrix.from_bcsr(rp, c, v, 2)
    for bad in (bm.LANES_ROW_OWNER, 3, 64 + 7):  # row owner needs bs >= 4; lanes are powers of two
        with pytest.raises(bm.BmfpError):
            m.set_lanes(bad)
    m.set_lanes(2)
    x = dev(np.ones(200))
    y = dev(np.zeros(200))
    m.spmv(x, y)
    m.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("bs", [2, 4, 8, 16, 32])
def test_column_owner_on_caller_arrays(lib, orc, cuda, bs, dtype):
    """bmfp_bcsr_spmv_colmajor on the transpose_blocks layout the caller holds."""
    import torch
    nbr = 2000 if bs <= 8 else 400
    rp, c, v = ragged_bcsr(nbr, nbr, bs, seed=bs + 70, dtype=dtype)
    x = np.random.default_rng(bs + 1).uniform(-1, 1, nbr * bs).astype(dtype)
    vt = bm.transpose_blocks(rp, v, bs)
    dy = torch.empty(nbr * bs, dtype=torch.float64 if dtype == np.float64 else torch.float32, device="cuda")
    bm.bcsr_spmv_colmajor(dev(rp), dev(c), dev(vt), dev(x), dy, bs)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    y_ref = orc.csr_spmv(crp, cc, cv, x, threads=8)
    assert np.all(np.abs(dy.cpu().numpy() - y_ref) <= spmv_tolerance(orc, crp, cc, cv, x, dtype))
