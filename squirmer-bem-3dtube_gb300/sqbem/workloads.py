"""Seeded synthetic workloads with the shapes and parameter distributions of the
five benchmark configurations (geometry only -- the reference's workloads are
generated meshes, there is no dataset).  Seed = 1000 + configuration index.

  duct       R = 1, L = 4, mu = 1, 24 x 24 x 6 panels (1680), dP in {0.5, 1, 2, 4}
  kinematics a/R = 0.3, beta = 0, level 3 (1280 panels), n_theta = 24, L/R = 4,
             B1 = 1, B2 = 0, towed drag
  sweep      128 instances: a/R ~ U[0.1, 0.6], beta ~ U[0, 0.8 (1 - a/R)],
             B2/B1 ~ U[-5, 5], level in {2, 3} with p = 1/2, n_theta = 24, L/R = 4
  adjoint    32 instances: a/R ~ U[0.2, 0.5], beta ~ U[0, 0.5], B2/B1 in {-3, 0, 3},
             level 2, n_theta = 24, L/R = 4
  ensemble   256 swimmers: a/R = 0.3, beta0 ~ U[0, 0.6], e uniform on the sphere,
             B2/B1 ~ U[-5, 5], level 2, n_theta = 24, L/R = 4; RK4, dt = 0.05,
             200 steps; field on a 25 x 25 x 41 grid per swimmer
"""
import numpy as np

SEED = 1000


def duct():
    return dict(R=1.0, L=4.0, mu=1.0, n_theta=24, n_z=24, n_r=6, dP=[0.5, 1.0, 2.0, 4.0])


def kinematics():
    return [dict(a_over_R=0.3, beta=0.0, L_over_R=4.0, e=(0.0, 0.0, 1.0), n_theta=24, n_r=4, sphere_level=3,
                 towed=1, alpha=0.0)]


def sweep(n=128, shard=0):
    """shard > 0 draws another independent set of n instances (replica k of a
    multi-GPU run); shard 0 is the benchmark set itself"""
    rng = np.random.default_rng(SEED + 2) if shard == 0 else np.random.default_rng([SEED + 2, shard])
    lam = rng.uniform(0.1, 0.6, n)
    beta = rng.uniform(0.0, 1.0, n) * 0.8 * (1.0 - lam)
    alpha = rng.uniform(-5.0, 5.0, n)
    level = np.where(rng.random(n) < 0.5, 2, 3)
    return [dict(a_over_R=float(lam[k]), beta=float(beta[k]), L_over_R=4.0, e=(0.0, 0.0, 1.0), n_theta=24, n_r=4,
                 sphere_level=int(level[k]), towed=0, alpha=float(alpha[k])) for k in range(n)]


def adjoint(n=32):
    rng = np.random.default_rng(SEED + 3)
    lam = rng.uniform(0.2, 0.5, n)
    beta = rng.uniform(0.0, 0.5, n)
    alpha = rng.choice([-3.0, 0.0, 3.0], n)
    return [dict(a_over_R=float(lam[k]), beta=float(beta[k]), L_over_R=4.0, e=(0.0, 0.0, 1.0), n_theta=24, n_r=4,
                 sphere_level=2, towed=0, alpha=float(alpha[k])) for k in range(n)]


def ensemble(n=256):
    rng = np.random.default_rng(SEED + 4)
    beta0 = rng.uniform(0.0, 0.6, n)
    e = rng.normal(size=(n, 3))
    e /= np.linalg.norm(e, axis=1)[:, None]
    alpha = rng.uniform(-5.0, 5.0, n)
    return [dict(a_over_R=0.3, beta0=float(beta0[k]), e=tuple(map(float, e[k])), alpha=float(alpha[k]),
                 sphere_level=2, n_theta=24, L_over_R=4.0, dt=0.05, steps=200) for k in range(n)]
