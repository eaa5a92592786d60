"""Device model generators against their host restatements, and a plan
built from a generated model equals one built from the same host arrays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_matlab_anticline_on_device_equals_host(built):
    from ela3d_gb300 import generate_model, media

    got = generate_model(media.matlab_spec(), 201, 201, 201)
    want = media.matlab_anticline()
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_dome_on_device_equals_host_restatement(built):
    from ela3d_gb300 import generate_model, media

    spec = media.anticline_256_spec(n=96, seed=3)
    got = generate_model(spec, 96, 80, 72)
    want = media.generate_host(spec, 96, 80, 72)
    for g, w in zip(got, want):
        ulp = np.abs(g.view(np.int32).astype(np.int64) - w.view(np.int32).astype(np.int64))
        assert ulp.max() <= 1 and (ulp == 0).mean() > 0.999


def test_plan_from_generated_model_equals_host_arrays(built):
    from ela3d_gb300 import Plan, configs, generate_model, media

    p, *_ = configs.anticline_256(nstep=40, n=64)
    spec = media.anticline_256_spec(n=64, seed=1)
    cp, cs, rho = generate_model(spec, 64, 64, 64)
    with Plan.from_model(p, spec) as a:
        a.run(40)
        sa = a.seismograms()
    with Plan(p, cp, cs, rho) as b:
        b.run(40)
        sb = b.seismograms()
    assert np.array_equal(sa, sb) and np.any(sa)


def test_server_request_with_generated_model(built):
    from ela3d_gb300 import Plan, Server, configs, media

    p, *_ = configs.anticline_256(nstep=30, n=48)
    spec = media.anticline_256_spec(n=48, seed=2)
    with Plan.from_model(p, spec, variant=0) as a:
        a.run(30)
        want = a.seismograms()
    with Server(variant=0) as srv:
        t = srv.submit_model(p, spec)
        srv.wait(t)
        assert np.array_equal(srv.read(t), want)
