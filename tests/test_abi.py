"""The C ABI boundary (include/pbt.h): the library loads, exports every
declared entry point, and rejects bad arguments before touching the GPU
(CPU only; no compute calls)."""
import ctypes as C
import re
import threading
from pathlib import Path

import pytest

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import _native as N

ROOT = Path(__file__).resolve().parents[1]


def declared(header: str) -> set[str]:
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(pbt_[a-z0-9_]+)\s*\(", text))


@pytest.mark.parametrize("header,loader", [("pbt.h", N.lib), ("pbt_batch.h", N.lib),
                                           ("pbt_shared.h", N.lib), ("pbt_synth.h", N.synth_lib)])
def test_every_declared_symbol_is_exported(header, loader):
    lib = loader()
    names = declared(header)
    assert len(names) >= 1
    for name in names:
        assert hasattr(lib, name), f"{name} declared in {header} but not exported"


def test_python_signatures_cover_header():
    assert declared("pbt.h") == set(N.SIGNATURES)
    assert declared("pbt_synth.h") == set(N.SYNTH_SIGNATURES)
    from pascal_btdma_gb300 import batch

    assert declared("pbt_batch.h") == set(batch.BATCH_SIGNATURES)
    from pascal_btdma_gb300 import shared

    assert declared("pbt_shared.h") == set(shared.SHARED_SIGNATURES)


def test_python_constants_match_header():
    """Status codes, precisions and flags in the ctypes layer equal pbt.h's."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "pbt.h").read_text(), flags=re.S)
    found = {}
    for name, val in re.findall(r"\b(PBT_[A-Z0-9_]+)\s*=\s*(\d+)", text):
        found[name] = int(val)
    for name, val in re.findall(r"#define\s+(PBT_FLAG_[A-Z_]+)\s+0x([0-9a-fA-F]+)u", text):
        found[name] = int(val, 16)
    assert {"PBT_ETIMEOUT", "PBT_ESINGULAR", "PBT_PREC_FF", "PBT_FLAG_DIRECT_LOADS"} <= set(found)
    for name, val in found.items():
        assert getattr(N, name) == val, name


def test_batch_create_rejects_without_gpu():
    import numpy as np

    from pascal_btdma_gb300 import batch

    with pytest.raises(ValueError, match="m=11"):
        batch.BatchPlan(np.array([2, 11]), np.array([10, 10]))
    with pytest.raises(ValueError, match="equal length"):
        batch.BatchPlan(np.array([2, 3]), np.array([10]))


def test_version_and_partition():
    assert N.lib().pbt_version() >= 100
    for n, p in [(128, 4), (10, 3), (2048, 8), (7, 7)]:
        firsts = [pbt.partition_1d(0, n - 1, p, r) for r in range(p)]
        assert firsts[0][0] == 0 and firsts[-1][1] == n - 1
        for (f0, l0), (f1, l1) in zip(firsts, firsts[1:]):
            assert f1 == l0 + 1 and (l0 - f0) >= (l1 - f1) >= (l0 - f0) - 1


def test_desc_defaults():
    d = N.PlanDesc()
    N.lib().pbt_plan_desc_init(C.byref(d))
    assert (d.nseg, d.precision, d.flags, d.max_iter) == (1, N.PBT_PREC_FP64, 0, 8)
    assert d.tol == 1e-12


def create(**kw):
    d = N.PlanDesc()
    N.lib().pbt_plan_desc_init(C.byref(d))
    base = dict(m=3, nsys=16, nrow=12, nseg=1)
    base.update(kw)
    for k, v in base.items():
        setattr(d, k, v)
    h = C.c_void_p()
    rc = N.lib().pbt_plan_create_ex(C.byref(h), C.byref(d))
    return rc, h, N.last_error()


@pytest.mark.parametrize(
    "kw,code,msg",
    [
        (dict(m=0), N.PBT_EINVAL, "block size"),
        (dict(m=11), N.PBT_EINVAL, "block size"),
        (dict(nsys=0), N.PBT_EINVAL, "nsys > 0"),
        (dict(nrow=1), N.PBT_EINVAL, "nrow >= 2"),
        (dict(nseg=0), N.PBT_EINVAL, "nseg"),
        (dict(nrow=8, nseg=3), N.PBT_EINVAL, "nseg"),
        (dict(nrow=10, nseg=4), N.PBT_EINVAL, ">= 3 rows"),
        (dict(flags=N.PBT_FLAG_CYCLIC, nrow=2), N.PBT_EINVAL, "nrow >= 3"),
        (dict(flags=N.PBT_FLAG_CYCLIC | N.PBT_FLAG_REFERENCE_METHOD), N.PBT_EINVAL, "nseg >= 2"),
        (dict(flags=0x100), N.PBT_EINVAL, "unknown flag"),
        (dict(flags=N.PBT_FLAG_DIRECT_LOADS | N.PBT_FLAG_STAGED_LOADS), N.PBT_EINVAL, "exclude each other"),
        (dict(flags=N.PBT_FLAG_CPU_LAYOUT | N.PBT_FLAG_INPLACE), N.PBT_EUNSUPPORTED, "CPU_LAYOUT"),
        (dict(threads_per_block=48), N.PBT_EINVAL, "threads_per_block"),
        (dict(precision=7), N.PBT_EUNSUPPORTED, "precision"),
        (dict(precision=N.PBT_PREC_FP32_REFINE, flags=N.PBT_FLAG_INPLACE), N.PBT_EINVAL, "unchanged"),
        (dict(precision=N.PBT_PREC_FP32_REFINE, nseg=2, flags=N.PBT_FLAG_CYCLIC), N.PBT_EUNSUPPORTED, "non-cyclic"),
        (dict(precision=N.PBT_PREC_FP32_REFINE, max_iter=0), N.PBT_EINVAL, "max_iter"),
    ],
)
def test_plan_create_rejects(kw, code, msg):
    rc, h, err = create(**kw)
    assert rc == code and not h.value
    assert msg in err


def test_null_plan_calls():
    lib = N.lib()
    assert lib.pbt_plan_destroy(None) == N.PBT_OK
    z = C.c_void_p(0)
    rc = lib.pbt_solve_noncyclic(None, z, z, z, z, 3, 16, 12, None)
    assert rc == N.PBT_ESTATE and "null plan" in N.last_error()
    assert lib.pbt_plan_status(None, None) == N.PBT_ESTATE
    assert lib.pbt_plan_workspace_bytes(None) == 0


def test_last_error_is_per_thread():
    create(m=0)
    seen = []
    t = threading.Thread(target=lambda: seen.append(N.last_error()))
    t.start()
    t.join()
    assert seen == [""] and "block size" in N.last_error()


def test_python_mirror_errors():
    plan = pbt.BtdmaGpuPlan()
    with pytest.raises(ValueError, match="block size"):
        plan.create(11, 16, 12)
    with pytest.raises(ValueError, match=">= 3 rows"):
        plan.create(3, 16, 10, nseg=4)
    with pytest.raises(ValueError, match="unknown precision"):
        plan.create(3, 16, 12, precision="fp16")
    with pytest.raises(RuntimeError, match="uncreated"):
        pbt.solve_noncyclic(plan, 0, 0, 0, 0, 3, 16, 12)
    assert not plan.created


def test_index_helpers_match_reference_layout():
    assert pbt.matrix_index(1, 2, 0, 1, 4, 5, 3) == 1 + 4 * (2 + 5 * (0 + 3 * 1))
    assert pbt.vector_index(3, 4, 2, 8, 6) == 3 + 8 * (4 + 6 * 2)


def test_cpu_layout_index_helpers_match_oracle_conversion():
    """pbt.cpu_matrix_index / cpu_vector_index agree with the oracle's layout
    conversion (the reference CPU layout a(m, m, nsys, n), d(m, nsys, n))."""
    import numpy as np

    from oracle import oracle as O

    m, nsys, nrow = 3, 5, 4
    g = np.arange(m * m * nsys * nrow, dtype=np.float64)
    c = O.gpu_to_cpu(m, nsys, nrow, True, g)
    gv = np.arange(m * nsys * nrow, dtype=np.float64)
    cv = O.gpu_to_cpu(m, nsys, nrow, False, gv)
    for sys, row, p, q in [(0, 0, 0, 0), (4, 3, 2, 1), (2, 1, 1, 2)]:
        assert c[pbt.cpu_matrix_index(sys, row, p, q, nsys, m)] == g[pbt.matrix_index(sys, row, p, q, nsys, nrow, m)]
        assert cv[pbt.cpu_vector_index(sys, row, p, nsys, m)] == gv[pbt.vector_index(sys, row, p, nsys, nrow)]


def test_shared_create_checks_before_the_gpu():
    """Bad sizes and a singular shared matrix are refused on the host."""
    import numpy as np

    from pascal_btdma_gb300 import shared

    with pytest.raises(ValueError):
        shared.SharedMatrix(11, 4, np.zeros(4 * 121), np.zeros(4 * 121), np.zeros(4 * 121))
    with pytest.raises(ValueError):
        shared.SharedMatrix(2, 4, np.zeros(3), np.zeros(16), np.zeros(16))
    m, nrow = 2, 4
    a, b, c = (np.zeros(nrow * m * m) for _ in range(3))  # B = 0: the first pivot is zero
    with pytest.raises(pbt.SingularBlockError):
        shared.SharedMatrix(m, nrow, a, b, c)
    with pytest.raises(ValueError):
        shared.SharedMatrix(m, nrow, a, b, c, precision="fp32_refine")
    # The C entry refuses other arithmetics itself, and float-float factors
    # beyond the float range (1/b = 1e40 here), before any device call.
    lib = shared._lib()
    h = C.c_void_p()
    one = np.ones(nrow * m * m)
    assert lib.pbt_shared_create(C.byref(h), m, nrow, one.ctypes.data, one.ctypes.data, one.ctypes.data,
                                 N.PBT_PREC_FP32_REFINE) == N.PBT_EUNSUPPORTED
    tiny, zero = np.full(2, 1e-40), np.zeros(2)
    assert lib.pbt_shared_create(C.byref(h), 1, 2, zero.ctypes.data, tiny.ctypes.data, tiny.ctypes.data,
                                 N.PBT_PREC_FF) == N.PBT_ERANGE
    assert not h.value


def test_heat3d_blocks_match_reference_stencil():
    """The heat3d blocks (build_matrix_kernel): interior rows hold the
    fourth-order stencil [-1, 16, -30, 16, -1]/12 scaled into sigma units."""
    import numpy as np

    from pascal_btdma_gb300 import shared

    nblk, sigma = 4, 0.1
    a, b, c = shared.heat3d_blocks(nblk, sigma)
    el = lambda x, q, i, j: x[q + nblk * (i + 2 * j)]  # noqa: E731
    q = 1  # interior: point 2q (i = 0) row of the assembled matrix, columns 2q-2 .. 2q+2
    row0 = [el(a, q, 0, 0), el(a, q, 0, 1), el(b, q, 0, 0), el(b, q, 0, 1), el(c, q, 0, 0), el(c, q, 0, 1)]
    assert np.allclose(row0, [sigma, -16 * sigma, 1 + 30 * sigma, -16 * sigma, sigma, 0.0])
    assert el(a, 0, 0, 0) == 0.0 and el(c, nblk - 1, 1, 1) == 0.0


def test_lines_helpers_and_host_checks():
    """pbt_lines from the host helpers, and the lines solve's checks that run
    before any device call."""
    import numpy as np

    from pascal_btdma_gb300 import shared

    L = pbt.Lines.packed(300, 64)
    assert (L.nsys_inner, L.nsys_outer, L.stride_inner, L.stride_outer, L.row_stride, L.elem_stride) == \
        (300, 1, 1, 0, 300, 300 * 64)
    # Lines of a C-ordered (6, 5, 4) array along each axis, blocks of 2 points.
    shape = (6, 5, 4)
    a = np.arange(np.prod(shape)).reshape(shape)
    for axis in range(3):
        if shape[axis] % 2:
            with pytest.raises(ValueError):
                shared.Lines.axis(shape, axis, 2)
            continue
        L = shared.Lines.axis(shape, axis, 2)
        flat = a.reshape(-1)
        others = [x for x in range(3) if x != axis]
        for s_out in range(L.nsys_outer):
            for s_in in range(L.nsys_inner):
                for q in range(shape[axis] // 2):
                    for i in range(2):
                        idx = [0, 0, 0]
                        idx[others[0]], idx[others[1]], idx[axis] = s_out, s_in, 2 * q + i
                        off = s_in * L.stride_inner + s_out * L.stride_outer + q * L.row_stride + i * L.elem_stride
                        assert flat[off] == a[tuple(idx)]
    # The C struct mirrors the header's field order.
    c = L.c()
    assert isinstance(c, N.Lines) and c.row_stride == L.row_stride
    with pytest.raises(RuntimeError):
        pbt.solve_noncyclic_lines(pbt.BtdmaGpuPlan(), None, None, None, None, L)


def test_strided_runner_lines_address_the_euler3d_layout():
    """The sweep runner's lines (python -m pascal_btdma_gb300.strided) address
    element e of point (i, j, k) of a C-ordered [e, k, j, i] array: rows along
    the sweep axis, lines over the other two."""
    import numpy as np

    from pascal_btdma_gb300 import strided

    n, E = 4, 3
    arr = np.arange(E * n ** 3).reshape(E, n, n, n)
    flat = arr.reshape(-1)
    for axis in "xyz":
        L = strided.lines_of(n, axis)
        for s_out in range(n):
            for s_in in range(n):
                for q in range(n):
                    for e in range(E):
                        off = s_in * L.stride_inner + s_out * L.stride_outer + q * L.row_stride + e * L.elem_stride
                        i, j, k = {"x": (q, s_in, s_out), "y": (s_in, q, s_out), "z": (s_in, s_out, q)}[axis]
                        assert flat[off] == arr[e, k, j, i]
    with pytest.raises(ValueError):
        strided.lines_of(n, "w")
