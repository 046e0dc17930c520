"""Host logic: case-file parsing and validation, data-file format, restart."""
import json
import struct

import numpy as np
import pytest

from microfc_gb300 import Case, cases, io, preprocess


def test_case_dict_round_trip_matches_builder():
    c = cases.shock_droplet_2d(nx=64, ny=32, steps=10)
    d = {"m": c.m, "n": c.n, "dt": c.dt, "t_step_start": 0, "t_step_stop": 10, "t_step_save": 10,
         "x_domain%beg": 0.0, "x_domain%end": 0.02, "y_domain%beg": 0.0, "y_domain%end": 0.01,
         "num_fluids": 2, "time_stepper": 3, "weno_order": 5, "weno_eps": 1e-16,
         "bc_x%beg": -3, "bc_x%end": -3, "bc_y%beg": -3, "bc_y%end": -3,
         "fluid_pp(1)%gamma": c.gammas[0], "fluid_pp(1)%pi_inf": c.pi_infs[0],
         "fluid_pp(2)%gamma": c.gammas[1], "fluid_pp(2)%pi_inf": c.pi_infs[1], "num_patches": 3}
    for i, p in enumerate(c.patches, start=1):
        d[f"patch_icpp({i})%geometry"] = p.geometry
        d[f"patch_icpp({i})%x_centroid"], d[f"patch_icpp({i})%y_centroid"] = p.centroid[:2]
        d[f"patch_icpp({i})%length_x"], d[f"patch_icpp({i})%length_y"] = p.length[:2]
        d[f"patch_icpp({i})%radius"] = p.radius
        d[f"patch_icpp({i})%smoothen"] = "T" if p.smoothen else "F"
        if p.smooth_patch_id:
            d[f"patch_icpp({i})%smooth_patch_id"] = p.smooth_patch_id
        d[f"patch_icpp({i})%smooth_coeff"] = p.smooth_coeff
        for a in p.alter_patch:
            d[f"patch_icpp({i})%alter_patch({a})"] = "T"
        for f in range(2):
            d[f"patch_icpp({i})%alpha_rho({f + 1})"] = p.alpha_rho[f]
            d[f"patch_icpp({i})%alpha({f + 1})"] = p.alpha[f]
        d[f"patch_icpp({i})%vel(1)"], d[f"patch_icpp({i})%vel(2)"] = p.vel[:2]
        d[f"patch_icpp({i})%pres"] = p.pres
    parsed = Case.from_dict(json.loads(json.dumps(d)))
    parsed.check()
    q_ref = preprocess.generate(c)[3]
    q_new = preprocess.generate(parsed)[3]
    assert np.array_equal(q_ref, q_new)
    nml = parsed.to_namelist()
    assert nml.startswith("&user_inputs") and "bc_y%end = -3" in nml and nml.rstrip().endswith("/")


@pytest.mark.parametrize("change,msg", [
    (dict(m=0), "Unsupported value of m"),
    (dict(dt=0.0), "Unsupported value of dt"),
    (dict(t_step_stop=0), "t_step_start and t_step_stop"),
    (dict(weno_order=4), "weno_order"),
    (dict(m=20), "m and weno_order"),
    (dict(weno_eps=1e-3), "weno_eps"),
    (dict(bc_x=(-1, -3)), "bc_x%beg and bc_x%end"),
    (dict(bc_y=(-3, -3)), "n and bc_y%beg"),
    (dict(gammas=(-1.0, 2.5)), "fluid_pp(i)%gamma"),
    (dict(weno_re_flux=True, re_shear=(10.0, 10.0), weno_order=3, m=199), "weno_Re_flux"),
])
def test_check_rejects_invalid_inputs_like_the_reference(change, msg):
    c = cases.sod_1d(m=99, steps=10, dt=1e-4).replace(**change)
    with pytest.raises(ValueError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        c.check()


def test_record_format_is_gfortran_sequential(tmp_path):
    a = np.arange(10, dtype=np.float64)
    p = tmp_path / "x.dat"
    io.write_record(str(p), a)
    raw = p.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == 80
    assert struct.unpack("<i", raw[-4:])[0] == 80
    assert np.array_equal(np.frombuffer(raw[4:-4], dtype="<f8"), a)
    assert np.array_equal(io.read_record(str(p)), a)


def test_subrecords_round_trip(tmp_path, monkeypatch):
    monkeypatch.setattr(io, "_MAX_SUB", 24)  # force splitting into 3-double sub-records
    a = np.arange(10, dtype=np.float64)
    p = tmp_path / "big.dat"
    io.write_record(str(p), a)
    raw = p.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == -24
    assert np.array_equal(io.read_record(str(p)), a)


def test_truncated_file_is_rejected(tmp_path):
    p = tmp_path / "t.dat"
    io.write_record(str(p), np.ones(4))
    p.write_bytes(p.read_bytes()[:-6])
    with pytest.raises(ValueError):
        io.read_record(str(p))


def test_data_files_round_trip_restart_layout(tmp_path):
    c = cases.shock_droplet_2d(nx=32, ny=16, steps=4)
    x_cb, y_cb, _, q = preprocess.generate(c)
    d = io.write_data_files(str(tmp_path), 0, c, q, x_cb, y_cb)
    assert d.endswith("p_all/p0/0")
    x2, y2, _, q2 = io.read_data_files(str(tmp_path), 0, c)
    assert np.array_equal(x2, x_cb) and np.array_equal(y2, y_cb) and np.array_equal(q2, q)
    with pytest.raises(FileNotFoundError):
        io.read_data_files(str(tmp_path), 7, c)
