"""Library runs: run_model (librarian/lib_tools.py:714-842), the model details (:845-943) and the
combined-library writer (librarian/combine.py:212-260)."""

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import sam_oracle as O


@pytest.mark.gpu
def test_model_details_match_reference(built_lib):
    from holodeck_gb300.librarian import lib_tools
    g = load_golden("ref_details.npz")
    edges = [g["mtot"], g["mrat"], g["redz"], g["fobs_edges"] / 2.0]
    gwb_pars, num_pars, gm, nm = lib_tools._calc_model_details(edges, g["redz_final"], g["number"])
    for ii in range(4):
        # strain-weighted: the device strain differs from the reference's in the last bits (1e-10)
        assert rel_err(gwb_pars[ii], g[f"gwb_params_{ii}"]) < 1e-9, ii
        assert rel_err(num_pars[ii], g[f"num_params_{ii}"]) < 1e-12, ii
    assert rel_err(gm, g["gwb_mtot_redz_final"]) < 1e-9
    assert rel_err(nm, g["num_mtot_redz_final"]) < 1e-12
    # against the oracle on the same inputs, including the redshift binning edge rule
    o = O.calc_model_details(edges, g["redz_final"], g["number"])
    assert np.array_equal(np.isnan(gm), np.isnan(o[2]))


@pytest.mark.gpu
def test_run_model_all_flags(built_lib):
    import holodeck_gb300 as H
    from holodeck_gb300 import constants as C
    from holodeck_gb300.librarian import lib_tools
    sam = H.sams.Semi_Analytic_Model(shape=(10, 11, 12), gpf=H.sams.GPF_Power_Law(), gmt=H.sams.GMT_Power_Law(),
                                     mmbulge=H.host_relations.MMBulge_KH2013(scatter_dex=0.0))
    hard = H.hardening.Fixed_Time_2PL_SAM(sam, 3.0 * C.GYR, rchar=100.0 * C.PC, gamma_inner=-1.0, gamma_outer=2.5)
    data = lib_tools.run_model(sam, hard, nfreqs=6, nreals=4, nloudest=2, gwb_flag=True, singles_flag=True,
                               details_flag=True, params_flag=True, seed=5)
    F = 6
    assert data["hc_ss"].shape == (F, 4, 2) and data["hc_bg"].shape == (F, 4)
    assert data["sspar"].shape == (4, F, 4, 2) and data["bgpar"].shape == (7, F, 4)
    assert data["gwb"].shape == (F, 4) and np.all(data["gwb"] > 0)
    assert [p.shape for p in data["gwb_params"]] == [(9, 11, F), (10, 11, F), (11, F), (11, F)]
    assert data["number"].shape == (9, 10, 11, F) and data["redz_final"].shape == (10, 11, 12, F)
    edges = [sam.mtot, sam.mrat, sam.redz, data["fobs_edges"] / 2.0]
    ref = lib_tools._calc_model_details(edges, data["redz_final"], data["number"])
    for a, b in zip(data["gwb_params"], ref[0]):
        assert np.array_equal(a, b, equal_nan=True)
    with pytest.raises(RuntimeError):
        lib_tools.run_model(sam, hard, gwb_flag=False, singles_flag=False)


def test_write_library_layout(tmp_path):
    """combine.py layout in npz: stacked sample outputs, NaN rows and parameters for failed samples."""
    from holodeck_gb300.librarian import lib_tools
    rng = np.random.default_rng(0)
    F, R, L = 3, 4, 2
    good = dict(fobs_cents=np.arange(F) + 1.0, fobs_edges=np.arange(F + 1) + 0.5, gwb=rng.random((F, R)),
                hc_ss=rng.random((F, R, L)), hc_bg=rng.random((F, R)), sspar=rng.random((4, F, R, L)),
                bgpar=rng.random((7, F, R)))
    samples = [good, None, good]
    params = rng.random((3, 2))
    path = lib_tools.write_library(tmp_path / "sam_lib.npz", samples, params, ["a", "b"], "PS_Test")
    with np.load(path) as lib:
        assert lib["gwb"].shape == (3, F, R) and lib["sspar"].shape == (3, 4, F, R, L)
        assert np.all(np.isnan(lib["gwb"][1])) and np.all(np.isnan(lib["sample_params"][1]))
        assert np.array_equal(lib["hc_bg"][2], good["hc_bg"])
        assert np.array_equal(lib["sample_params"][0], params[0])
        assert list(lib["attr_param_names"].astype(str)) == ["a", "b"]
        assert str(lib["attr_parameter_space_class_name"]) == "PS_Test"
