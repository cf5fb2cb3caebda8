"""GPU: rt_scene_add_things builds the same scene as one rt_scene_add_thing per thing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_add_things_equals_add_thing_loop(product, cuda):
    R = product
    sp = R.rtow_spheres(R.RT_RECIPE_GLIBC, 1, 11)
    m = R.Scene()
    v, i = m.get_mesh(m.add_sphere_mesh(1.0, 2))
    m.close()
    opts, T = [], []
    for c, r_, t_, a_, f_, i_ in zip(sp["centers"], sp["radii"], sp["types"], sp["albedos"], sp["fuzz"], sp["index"]):
        opts.append(R.optics(int(t_), a_, float(f_), float(i_)))
        T.append([r_, 0, 0, c[0], 0, r_, 0, c[1], 0, 0, r_, c[2]])
    T = np.asarray(T, np.float32)
    one, bulk = R.Scene(), R.Scene()
    m1, m2 = one.add_mesh(v, i), bulk.add_mesh(v, i)
    ids1 = [one.add_thing(o, m1, t) for o, t in zip(opts, T)]
    ids2 = bulk.add_things(opts, [m2] * len(opts), T)
    assert ids1 == ids2 == list(range(len(opts)))
    for k in (0, 17, len(opts) - 1):
        assert np.array_equal(one.get_transform(k)[1], bulk.get_transform(k)[1])
    one.build(60)
    bulk.build(60)
    w, h = 96, 64
    cam, params = R.rtow_camera(w, h), R.launch_params(w, h, 2, depth=16, seed=4)
    a, b = R.render(one, cam, params), R.render(bulk, cam, params)
    assert np.array_equal(a["rawRGB"].view(np.uint32), b["rawRGB"].view(np.uint32))
    assert np.array_equal(a["rpp"], b["rpp"])
    one.close()
    bulk.close()
