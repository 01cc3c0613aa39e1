"""CPU checks of the benchmark/test tooling beside the product library: the
generator and probe libraries build and export what esp_workloads.h
declares, none of it is in the product library, and the oracle's build of
the generators (the benchmark's reference arm) makes the same bytes."""
import ctypes

import numpy as np

import oracle as O
import workloads as W
from esperanto_gb300 import _native as N
from esperanto_gb300 import build


def test_tooling_libraries_export_their_header():
    names = W.declared_symbols()
    assert len(names) == 10
    synth = ctypes.CDLL(W.build_synth())
    probe = ctypes.CDLL(W.build_probe())
    for n in names:
        lib = probe if n.startswith("esp_probe") else synth
        assert hasattr(lib, n), n


def test_product_library_holds_no_tooling():
    lib = ctypes.CDLL(build.build())
    for n in W.declared_symbols() + ["esp_int_peaks", "esp_simd16_peaks"]:
        assert not hasattr(lib, n), n
    assert not set(W.declared_symbols()) & set(N.exported_symbols())


def test_oracle_build_of_generators_makes_the_same_bytes():
    ol = O.synth_lib()
    for shape, n in ((0, 3000), (2, 5000)):
        a, p = W.synth_gotoh(3, n, shape)
        b, q = W.synth_gotoh(3, n, shape, lib=ol)
        assert (a == b).all() and (p == q).all()
    a, p = W.synth_myers(2, 4000)
    b, q = W.synth_myers(2, 4000, lib=ol)
    assert (a == b).all() and (p == q).all()
    x = W.synth_splice(4, 300)
    y = W.synth_splice(4, 300, lib=ol)
    assert all((u == v).all() for u, v in zip(x, y))
    g1, c1 = W.synth_genome(5, 1_000_000, 3)
    g2, c2 = W.synth_genome(5, 1_000_000, 3, lib=ol)
    assert (g1 == g2).all() and (c1 == c2).all()
    r1 = W.synth_request(5, 1, g1, c1, 999)
    r2 = W.synth_request(5, 1, g2, c2, 999, lib=ol)
    assert all((u == v).all() for u, v in zip(r1, r2))


def test_generators_are_seeded_and_thread_independent():
    a, p = W.synth_gotoh(9, 10000, 2)
    b, q = W.synth_gotoh(9, 10000, 2)
    assert (a == b).all() and (p == q).all()
    # a prefix of a workload is the smaller workload of the same seed
    c, r = W.synth_gotoh(9, 2000, 2)
    assert (r["read_len"] == p["read_len"][:2000]).all()
    assert np.array_equal(r["band_half"], p["band_half"][:2000])
