"""Tile plans (bsa_gpu_setTilePlan / loadTilePlans / getTilePlan): the table the autotuner
writes is parsed by the library, the first matching plan wins, values that do not fit a case
fall back to the default rule.  Host logic only (no GPU)."""
import pytest

from bsalib_gb300 import api


@pytest.fixture
def lib():
    lib = api.load()
    yield lib
    lib.bsa_gpu_loadTilePlans(None)   # the packaged table again
    lib.bsa_Finalise()


def test_defaults_are_the_narrowest_widths(lib):
    assert lib.bsa_gpu_clearTilePlans() == 0
    assert [api.tile_plan(api.PLAN_CLS_E_WIDTH, n, 800, 513) for n in (4, 12, 20, 30, 40)] == [8, 16, 24, 32, 48]
    assert [api.tile_plan(api.PLAN_CLS_D_WIDTH, n, 800, 513) for n in (4, 12, 20, 30, 40)] == [8, 16, 24, 32, 64]
    assert [api.tile_plan(api.PLAN_MSH_WIDTH, n, 800) for n in (4, 12, 20, 60)] == [8, 16, 24, 64]
    assert api.tile_plan(api.PLAN_CLS_FORM, 24, 800, 513) == 1
    # E form mode passes: 8 one, 24 two, 16 two on grids above 700 points per axis, 32 / 48 two
    assert [api.tile_plan(api.PLAN_CLS_E_SPLIT, n, 800, 513) for n in (4, 12, 20, 30, 40)] == [1, 1, 2, 2, 2]
    assert [api.tile_plan(api.PLAN_CLS_E_SPLIT, n, 800, 1025) for n in (4, 12, 20)] == [1, 2, 2]


def test_table_file_first_match_and_fallbacks(lib, tmp_path):
    f = tmp_path / "plans.txt"
    f.write_text("# a comment\n"
                 "cls_e_width 9 16 0 1000 0 300 24   # measured\n"
                 "cls_e_width 9 16 0 100000 0 100000 32\n"
                 "cls_d_width 1 8 0 100000 0 100000 12\n"        # not a built width: default
                 "cls_form 25 48 0 100000 301 100000 0\n"
                 "msh_width 17 24 0 100000 0 100000 16\n"          # narrower than the modes: default
                 "msh_width 1 8 0 100000 0 100000 24\n"
                 "cls_e_split 17 24 0 100000 0 100000 1\n"
                 "cls_e_split 9 16 0 100000 0 100000 3\n")         # not 1 or 2: default
    assert lib.bsa_gpu_loadTilePlans(str(f).encode()) == 0
    assert api.tile_plan(api.PLAN_CLS_E_WIDTH, 12, 500, 129) == 24
    assert api.tile_plan(api.PLAN_CLS_E_WIDTH, 12, 5000, 129) == 32
    assert api.tile_plan(api.PLAN_CLS_E_WIDTH, 20, 500, 129) == 24      # no plan: default
    assert api.tile_plan(api.PLAN_CLS_D_WIDTH, 6, 500, 129) == 8
    assert api.tile_plan(api.PLAN_CLS_FORM, 30, 500, 513) == 0
    assert api.tile_plan(api.PLAN_CLS_FORM, 30, 500, 129) == 1
    assert api.tile_plan(api.PLAN_MSH_WIDTH, 20, 500) == 24
    assert api.tile_plan(api.PLAN_MSH_WIDTH, 6, 500) == 24
    assert api.tile_plan(api.PLAN_CLS_E_SPLIT, 20, 500, 129) == 1
    assert api.tile_plan(api.PLAN_CLS_E_SPLIT, 12, 500, 1025) == 2
    assert api.tile_plan(api.PLAN_CLS_E_SPLIT, 30, 500, 129) == 2          # width 32: always two
    # a plan set through the C-ABI goes ahead of the table
    assert lib.bsa_gpu_setTilePlan(api.PLAN_CLS_E_WIDTH, 1, 64, 0, 1 << 30, 0, 1 << 30, 48) == 0
    assert api.tile_plan(api.PLAN_CLS_E_WIDTH, 12, 500, 129) == 48


def test_bad_table_is_refused(lib, tmp_path):
    f = tmp_path / "bad.txt"
    f.write_text("cls_e_width 1 8 0 10\n")
    assert lib.bsa_gpu_loadTilePlans(str(f).encode()) == -1   # BSA_ERR_ARG
    assert b"bad plan on line 1" in lib.bsa_lastError()


def test_packaged_table_parses(lib):
    import os
    path = os.path.join(os.path.dirname(api.__file__), "data", "tile_plans.txt")
    if not os.path.exists(path):
        pytest.skip("no packaged tile plans")
    assert lib.bsa_gpu_loadTilePlans(path.encode()) == 0
