"""CPU checks that the seeded synthetic maps follow the workload definition:
sky gradient 2.0 at the horizon to 0.5 at the poles, one log-normal(0, 1)
factor per texel, 8 Gaussian suns of 1-3 degrees with radiance log-uniform in
[1, sun_max], alpha 1 -- and that sun_params replays make_env's draws."""
import numpy as np
import pytest

from althea_gb300 import synth


def test_sky_gradient_and_noise_statistics():
    w, h = 1024, 512
    env = synth.make_env(w, h, seed=3, with_suns=False)
    assert env.dtype == np.float32 and env.shape == (h, w, 4)
    assert np.all(env[..., 3] == 1.0)
    assert np.array_equal(env[..., 0], env[..., 1]) and np.array_equal(env[..., 1], env[..., 2])
    pitch = np.pi * ((np.arange(h) + 0.5) / h - 0.5)
    sky = 2.0 + (0.5 - 2.0) * np.abs(np.sin(pitch))
    z = np.log(env[..., 0] / sky[:, None].astype(np.float32))
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01  # log-normal(0, 1)
    assert sky[h // 2] > 1.99 and sky[0] < 0.51  # horizon 2.0, poles 0.5


def test_same_seed_same_map_other_seed_other_map():
    a = synth.make_env(64, 32, seed=11, sun_max=1e6)
    assert np.array_equal(a, synth.make_env(64, 32, seed=11, sun_max=1e6))
    assert not np.array_equal(a, synth.make_env(64, 32, seed=12, sun_max=1e6))


@pytest.mark.parametrize("sun_max", [1e4, 1e6])
def test_suns_follow_their_parameters(sun_max):
    w, h, seed = 512, 256, 5
    suns = synth.sun_params(w, h, seed=seed, sun_max=sun_max)
    assert len(suns) == 8
    for d, sigma, lum in suns:
        assert abs(np.linalg.norm(d) - 1.0) < 1e-12
        assert np.deg2rad(1.0) <= sigma <= np.deg2rad(3.0)
        assert 1.0 <= lum <= sun_max
    # the suns are the difference to the sun-free map, texel for texel
    env = synth.make_env(w, h, seed=seed, sun_max=sun_max).astype(np.float64)
    base = synth.make_env(w, h, seed=seed, with_suns=False).astype(np.float64)
    dirs = synth.texel_directions(w, h)
    model = sum(lum * np.exp(-np.arccos(np.clip(dirs @ d, -1, 1)) ** 2 / (2 * sigma ** 2))
                for d, sigma, lum in suns)
    diff = env[..., 0] - base[..., 0]
    assert np.allclose(diff, model, rtol=1e-5, atol=1e-4 * (1 + base[..., 0]))
