"""CPU tests of libacqgb300's host side through its C ABI (no GPU needed).

The library must load here, export every symbol include/acqgb300.h declares, and agree with
the oracle on geometry, validation, code generation and the CFAR threshold.
"""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import _lib as L
from oracle import acq_oracle as O
from oracle import gnss_codes as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SYS = {"GPSL1CA": (A.GPSL1CA(), G.GPSL1CA), "GPSL5I": (A.GPSL5I(), G.GPSL5I),
       "GalileoE1B": (A.GalileoE1B(), G.GalileoE1B)}


def test_library_exports_every_header_symbol():
    header = open(os.path.join(ROOT, "include", "acqgb300.h")).read()
    declared = set(re.findall(r"\b(acq_[a-z_0-9]+)\s*\(", header))
    assert declared, "no declarations parsed"
    lib = C.CDLL(L.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(L.EXPORTED) == declared, set(L.EXPORTED) ^ declared
    assert b"sm_103a" in L.load().acq_version()


def test_python_option_constants_match_the_header():
    header = open(os.path.join(ROOT, "include", "acqgb300.h")).read()
    defines = dict(re.findall(r"#define (ACQ_(?:OPT|TILE|FORM|PREC)_\w+)\s+(-?\d+)", header))
    from acqgb300 import api
    for name, val in defines.items():
        if name.startswith("ACQ_PREC_"):
            assert api.PRECISIONS[name[len("ACQ_PREC_"):].lower()] == int(val), name
        else:
            assert getattr(L, name) == int(val), name


def test_julia_option_table_matches_the_header():
    header = open(os.path.join(ROOT, "include", "acqgb300.h")).read()
    opts = {name: int(v) for name, v in re.findall(r"#define ACQ_OPT_(\w+)\s+(-?\d+)", header)}
    jl = open(os.path.join(ROOT, "acquisition.jl_gb300", "julia", "AcquisitionGB300.jl")).read()
    table = jl[jl.index("const OPTIONS = Dict("):]
    table = table[:table.index(")\n")]
    got = {name.upper(): int(v) for name, v in re.findall(r":(\w+) => (\d+)", table)}
    assert got == opts, set(got.items()) ^ set(opts.items())


_C_SIZE = {"int32_t": 4, "uint32_t": 4, "int64_t": 8, "double": 8, "float": 4}
_JL_SIZE = {"Int32": 4, "UInt32": 4, "Int64": 8, "Float64": 8, "Float32": 4}


def _c_structs(header):
    out = {}
    for body, name in re.findall(r"typedef struct \{(.*?)\} (\w+);", header, re.S):
        fields = []
        for line in re.sub(r"/\*.*?\*/", "", body, flags=re.S).split(";"):
            line = line.strip()
            if not line:
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s*(\*?)\s*(.*)", line)
            typ, ptr, names = m.groups()
            for nm in names.split(","):
                nm = nm.strip().lstrip("*")
                arr = re.match(r"(\w+)\[(\d+)\]", nm)
                if arr:
                    fields.append((arr.group(1), _C_SIZE[typ] * int(arr.group(2))))
                else:
                    fields.append((nm, 8 if ptr or "*" in names else _C_SIZE[typ]))
        out[name] = fields
    return out


def _jl_struct(src, name):
    """(field, bytes) of a plain-bits Julia struct of the binding."""
    body = re.search(r"^struct %s\b[^\n]*\n(.*?)\nend" % name, src, re.S | re.M).group(1)
    fields = []
    for fname, typ in re.findall(r"^\s*(\w+)::(\S+)", body, re.M):
        tup = re.match(r"NTuple\{(\d+),(\w+)\}", typ)
        size = 8 if typ.startswith("Ptr{") else _JL_SIZE[tup.group(2)] * int(tup.group(1)) if tup else _JL_SIZE[typ]
        fields.append((fname, size))
    return fields


def test_julia_binding_matches_the_header():
    # the ccall module a maintainer of Acquisition.jl would add (not executed here: no Julia):
    # its structs have the header's fields in the header's order and sizes, every symbol it
    # calls is declared, and it binds the acquire path, the detection helpers and the batch API
    header = open(os.path.join(ROOT, "include", "acqgb300.h")).read()
    jl = open(os.path.join(ROOT, "acquisition.jl_gb300", "julia", "AcquisitionGB300.jl")).read()
    c = _c_structs(header)
    for jname, cname in [("PlanDesc", "acq_plan_desc"), ("Geometry", "acq_geometry"), ("CResult", "acq_result"),
                         ("BatchItem", "acq_batch_item"), ("CorrCell", "acq_corr_cell"),
                         ("CorrResult", "acq_corr_result")]:
        assert _jl_struct(jl, jname) == c[cname], (jname, _jl_struct(jl, jname), c[cname])
    declared = set(re.findall(r"\b(acq_\w+)\s*\(", header))
    called = set(re.findall(r"ccall\(\(:(acq_\w+), lib\)", jl))
    assert called <= declared, called - declared
    assert {"acq_plan_create", "acq_plan_destroy", "acq_plan_get_geometry", "acq_acquire", "acq_cfar_threshold",
            "acq_plan_set_option", "acq_plan_get_option", "acq_batch_create", "acq_batch_run", "acq_batch_destroy",
            "acq_last_error"} <= called
    for name in ("plan_acquire", "acquire!", "acquire", "is_detected", "get_num_cells", "cfar_threshold"):
        assert re.search(r"^(function )?%s\(" % re.escape(name), jl, re.M), name
    # the 15 fields of the reference's AcquisitionResults (src/Acquisition.jl:81-109), in order
    res = re.search(r"^struct AcquisitionResults\{S,D<:AbstractRange\}\n(.*?)\nend", jl, re.S | re.M).group(1)
    assert re.findall(r"^\s*(\w+)::", res, re.M) == [
        "system", "prn", "sampling_frequency", "carrier_doppler", "code_phase", "secondary_code_phase", "CN0",
        "noise_power", "peak_to_noise_ratio", "num_noncoherent_integrations", "power_bins", "dopplers", "num_blocks",
        "block_size", "num_secondary_rotations"]


def test_python_binding_structs_match_the_header():
    # the ctypes structures the Python package passes through the C ABI: the header's fields, in
    # order, with the header's sizes
    from acqgb300 import batch as B
    header = open(os.path.join(ROOT, "include", "acqgb300.h")).read()
    c = _c_structs(header)
    for cls, cname in [(L.PlanDesc, "acq_plan_desc"), (L.Geometry, "acq_geometry"), (L.Result, "acq_result"),
                       (L.NoiseStats, "acq_noise_stats"), (L.SynthSat, "acq_synth_sat"), (L.CorrCell, "acq_corr_cell"),
                       (L.CorrResult, "acq_corr_result"), (B.BatchItemC, "acq_batch_item")]:
        got = [(name, C.sizeof(typ)) for name, typ in cls._fields_]
        assert got == c[cname], (cname, got, c[cname])


def test_result_struct_layout():
    assert C.sizeof(L.Result) == 72
    assert C.sizeof(L.PlanDesc) == 56


CONFIGS = [
    ("GPSL1CA", 4e6, 7000, 1, 1, 1), ("GPSL1CA", 5e6, 5000, 10, 1, 8), ("GPSL1CA", 5e6, 5000, 40, 1, 2),
    ("GPSL1CA", 5e6, 5000, 40, 4, 2), ("GPSL1CA", 5e6, 5000, 10, 2, 8), ("GPSL1CA", 2.048e6, 10000, 40, 4, 5),
    ("GPSL1CA", 16.368e6, 5000, 5, 1, 1), ("GPSL1CA", 16.368e6, 5000, 3, 3, 1), ("GPSL1CA", 10e6, 7000, 20, 1, 1),
    ("GPSL1CA", 1.542e6, 7000, 1, 1, 1), ("GPSL5I", 20e6, 10000, 20, 1, 4), ("GPSL5I", 20e6, 10000, 20, 2, 4),
    ("GPSL5I", 25e6, 8000, 10, 1, 1), ("GPSL5I", 10.24e6, 1000, 10, 1, 1), ("GPSL5I", 12e6, 7000, 1, 1, 3),
    ("GalileoE1B", 12e6, 8000, 1, 1, 1), ("GalileoE1B", 12e6, 8000, 1, 1, 5),
]


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "-".join(map(str, c)))
def test_geometry_matches_oracle(cfg):
    name, fs, cov, n_coh, n_be, n_nc = cfg
    a_sys, o_sys = SYS[name]
    g = A.plan_geometry(a_sys, fs, min_doppler_coverage=cov, num_coherently_integrated_code_periods=n_coh,
                        bit_edge_search_steps=n_be, num_noncoherent_accumulations=n_nc)
    o = O.plan_geometry(o_sys, fs, cov, n_coh, n_be, n_nc)
    assert (g.samples_per_code, g.samples_per_code_eff, g.num_blocks, g.block_size, g.fft_size, g.num_data_bits,
            g.num_doppler_bins, g.num_secondary_rotations) == (o["spc"], o["spc_eff"], o["nb"], o["bs"], o["F"],
                                                               o["ndb"], o["ndop"], o["R"])
    assert g.doppler_first_hz == o["freqs"][0] and g.doppler_step_hz == o["step"]
    thr = O.cfar_threshold(0.01, o["ndop"] * o["spc"] * o["R"], n_nc)
    assert g.cfar_threshold_pfa001 == pytest.approx(thr, rel=1e-10)


BAD = [dict(num_coherently_integrated_code_periods=30), dict(num_coherently_integrated_code_periods=20,
       bit_edge_search_steps=3), dict(bit_edge_search_steps=2), dict(num_noncoherent_accumulations=0),
       dict(num_coherently_integrated_code_periods=0), dict(bit_edge_search_steps=0),
       dict(min_doppler_coverage=1.1e6)]


@pytest.mark.parametrize("kw", BAD)
def test_validation_errors_match_oracle(kw):
    with pytest.raises(A.ArgumentError):
        A.plan_geometry(A.GPSL1CA(), 2.048e6, **kw)
    okw = dict(min_doppler_coverage=kw.get("min_doppler_coverage", 7000.0),
               n_coh=kw.get("num_coherently_integrated_code_periods", 1), n_be=kw.get("bit_edge_search_steps", 1),
               n_nc=kw.get("num_noncoherent_accumulations", 1))
    with pytest.raises(O.ArgumentError):
        O.plan_geometry(G.GPSL1CA, 2.048e6, **okw)


def test_secondary_code_error_messages():
    # test/plan.jl:70-121 text checks
    with pytest.raises(A.ArgumentError) as e:
        A.plan_geometry(A.GPSL5I(), 10.24e6, min_doppler_coverage=1000, num_coherently_integrated_code_periods=5)
    m = str(e.value)
    for s in ("secondary", "5", "10", "68", "num_coherently_integrated_code_periods",
              "num_noncoherent_accumulations", "use_secondary_code"):
        assert s in m
    with pytest.raises(A.ArgumentError) as e:
        A.plan_geometry(A.GPSL5I(), 10.24e6, min_doppler_coverage=1000, num_coherently_integrated_code_periods=10,
                        max_secondary_code_rotations=8)
    assert "max_secondary_code_rotations" in str(e.value) and "GPSL5I" in str(e.value)
    g = A.plan_geometry(A.GPSL5I(), 10.24e6, min_doppler_coverage=1000, num_coherently_integrated_code_periods=5,
                        use_secondary_code=False)
    assert g.num_secondary_rotations == 1


@pytest.mark.parametrize("name,fs,fc_off,start", [
    ("GPSL1CA", 4e6, 0.0, 0.0), ("GPSL1CA", 5e6, 0.0, 300.5), ("GPSL1CA", 10e6, 0.81, 123.456),
    ("GPSL5I", 10.24e6, 0.0, 0.0), ("GPSL5I", 20e6, 7.8, 5115.3), ("GPSL5I", 25e6, 0.0, 0.0),
    ("GalileoE1B", 12e6, 0.0, 0.0), ("GalileoE1B", 12e6, 1.1, 2000.25)])
def test_gen_code_matches_oracle(name, fs, fc_off, start):
    a_sys, o_sys = SYS[name]
    n = 3 * int(math.ceil(o_sys.code_length / o_sys.code_freq * fs))
    for prn in (1, 7, 32):
        fc = o_sys.code_freq + fc_off
        a = a_sys.gen_code(n, prn, fs, fc, start)
        o = G.gen_code(n, o_sys, prn, fs, fc, start)
        assert np.array_equal(a, o), (name, prn)


def test_gen_code_l5i_all_prns_and_l1_all_prns():
    for prn in range(1, 38):
        assert np.array_equal(A.GPSL5I().gen_code(10230, prn, 10.23e6), G.GPSL5I.full_chips(prn)[:10230])
    for prn in range(1, 33):
        assert np.array_equal(A.GPSL1CA().gen_code(1023, prn, 1.023e6), G.l1ca_chips(prn))


@pytest.mark.parametrize("M", [1, 2, 3, 4, 8, 16])
def test_cfar_threshold_matches_scipy(M):
    for pfa in (0.1, 0.01, 1e-3):
        for cells in (1, 100, 10_000, 1_000_000, 100_000_000, 2_000_000_000):
            assert A.cfar_threshold(pfa, cells, M) == pytest.approx(O.cfar_threshold(pfa, cells, M), rel=1e-9)
    assert A.cfar_threshold(0.01, 1) == pytest.approx(-math.log(0.01), rel=1e-12)


@pytest.mark.parametrize("system,fs,n_coh,rotations", [("GPSL5I", 12e6, 10, 10), ("GPSL1CA", 2.048e6, 1, 1)])
def test_num_cells_count_the_rotation_expansion(system, fs, n_coh, rotations):
    # src/Acquisition.jl:124-142 (issue #70, test/secondary_code_search.jl:473-530): on the rotation
    # path the peak is taken over num_secondary_rotations times the Doppler x code-phase cells,
    # get_num_cells counts them, and is_detected flips exactly at the threshold for that count;
    # off the rotation path the count is the bare grid
    from types import SimpleNamespace
    plan = O.plan_acquire(SYS[system][1], fs, [1], num_coherently_integrated_code_periods=n_coh, precision="f32")
    assert plan.num_secondary_rotations == rotations
    ndop, spc = plan.num_doppler_bins, plan.num_blocks * plan.block_size
    r = SimpleNamespace(dopplers=np.zeros(ndop), num_blocks=plan.num_blocks, block_size=plan.block_size,
                        num_secondary_rotations=plan.num_secondary_rotations, num_noncoherent_integrations=1,
                        peak_to_noise_ratio=0.0)
    assert A.get_num_cells(r) == rotations * ndop * spc
    thr = A.cfar_threshold(0.01, A.get_num_cells(r), num_noncoherent_integrations=1)
    assert thr > A.cfar_threshold(0.01, ndop * spc) or rotations == 1
    r.peak_to_noise_ratio = np.float32(thr * (1 + 1e-6))
    assert A.is_detected(r, pfa=0.01)
    r.peak_to_noise_ratio = np.float32(thr * (1 - 1e-6))
    assert not A.is_detected(r, pfa=0.01)


def test_cfar_argument_errors():
    for bad in [(0.0, 100), (1.0, 100), (-0.1, 100), (0.01, 0)]:
        with pytest.raises(A.ArgumentError):
            A.cfar_threshold(*bad)
    with pytest.raises(A.ArgumentError):
        A.cfar_threshold(0.01, 100, 0)


def test_plan_create_fails_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(A.AcquisitionError):
        A.plan_acquire(A.GPSL1CA(), 4e6, [1])


def test_correlator_create_fails_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = L.load()
    h = C.c_void_p()
    prns = (C.c_int32 * 2)(1, 2)
    st = lib.acq_corr_create(L.ACQ_GPS_L1CA, 10e6, prns, 2, None, C.byref(h))
    assert st == L.ACQ_ERR_CUDA and h.value is None
    bad = (C.c_int32 * 1)(40)
    assert lib.acq_corr_create(L.ACQ_GPS_L1CA, 10e6, bad, 1, None, C.byref(h)) == L.ACQ_ERR_ARGUMENT
    assert "PRN must be in 1:32" in L.last_error()


@pytest.mark.parametrize("nb,bs,width,fs", [(4, 8, 32, 1.023e6 * 32 / 1023), (16, 128, 2048, 2.048e6),
                                             (20, 250, 5000, 5e6), (25, 800, 200000, 20e6), (16, 250, 4000, 4e6)])
def test_chip_order_matches_oracle(nb, bs, width, fs):
    perm, axis = A.chip_order(nb, bs, width, 1.023e6, fs)
    dummy = np.arange(width, dtype=np.float32)[None, :]
    o_axis, o_sorted, o_order = O.fmdbzp_sort_by_chip(dummy, nb, bs, 1.023e6, fs)
    assert np.array_equal(perm, o_order)
    assert np.array_equal(axis, o_axis)
    # test/plot.jl:56-76 properties: monotone, within [0, code_length), unique
    assert np.all(np.diff(axis) >= 0) and axis.min() >= 0 and axis.max() < width * 1.023e6 / fs
    if width == nb * bs:      # one code period: a bijection (rotation surfaces repeat every period)
        assert len(np.unique(axis)) == width


def test_column_to_tau_known_answers():
    # test/plot.jl:18-41
    assert [O.fmdbzp_column_to_tau(c, 4, 8) for c in (0, 1, 8, 16, 24)] == [0, 1, 24, 16, 8]
    assert O.fmdbzp_column_to_tau(0, 32, 64) == 0
    assert sorted(O.fmdbzp_column_to_tau(c, 4, 8) for c in range(32)) == list(range(32))


def test_bounded_wait_selftest_fails_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    st = C.c_int32(-1)
    assert L.load().acq_selftest_bounded_wait(0, 1000, C.byref(st)) == L.ACQ_ERR_CUDA
    assert L.load().acq_selftest_bounded_wait(0, 0, C.byref(st)) == L.ACQ_ERR_ARGUMENT
