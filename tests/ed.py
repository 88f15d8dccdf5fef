"""Exact diagonalisation for small MagnetModel lattices (restatement of
test/ed/ed.jl and test/ed/magnet.jl) and the binning/jackknife statistics
used to compare Monte Carlo estimates with it (test/test_ed_compare.jl)."""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


class Lifter:
    """test/ed/ed.jl:6-21 -- site 1 is the slowest index of the product basis."""

    def __init__(self, dims):
        self.dims = list(dims)
        self.cum = [1] + list(np.cumprod(self.dims))

    def lift(self, pos, op):
        dl = int(self.cum[pos - 1])
        dr = int(self.cum[-1] // self.cum[pos])
        return sp.kron(sp.kron(sp.identity(dl, format="csr"), sp.csr_matrix(op)), sp.identity(dr, format="csr"), format="csr")

    def spin(self, S, pos, idx):
        sp, sz = S.spin_operators(self.dims[pos - 1])
        if idx == 1:
            return self.lift(pos, 0.5 * (sp + sp.T))
        if idx == 2:
            return self.lift(pos, 0.5j * (sp - sp.T))
        return self.lift(pos, sz)


def hamiltonian(S, model):
    """test/ed/magnet.jl:10-25."""
    lif = Lifter(model.site_spin_states)
    D = int(lif.cum[-1])
    H = sp.csr_matrix((D, D))
    for bond, p in zip(model.lattice.bonds, model.bond_params):
        i, j = bond.i, bond.j
        heis = sum(lif.spin(S, i, a) @ lif.spin(S, j, a) for a in (1, 2, 3)).real
        H = H + p.J * heis + p.J * p.d * lif.spin(S, i, 3) @ lif.spin(S, j, 3)
        H = H + p.hz[0] * lif.spin(S, i, 3) + p.hz[1] * lif.spin(S, j, 3)
        sxi = lif.spin(S, i, 1).real
        sxj = lif.spin(S, j, 1).real
        H = H + p.Dx[0] * sxi @ sxi + p.Dx[1] * sxj @ sxj
        szi = lif.spin(S, i, 3)
        szj = lif.spin(S, j, 3)
        H = H + p.Dz[0] * szi @ szi + p.Dz[1] * szj @ szj
    return H.toarray(), lif


def ed_observables(S, model, Ts):
    """test/ed/ed.jl:49-72 and 121-157 (ensemble averages, energy and specific heat) and test/ed/magnet.jl:27-97 (magnetisation estimators)."""
    H, lif = hamiltonian(S, model)
    Es, psi = np.linalg.eigh(H)
    Ts = np.asarray(Ts, dtype=float)
    Enorm = Es - Es.min()
    rho = np.exp(-Enorm[:, None] / Ts[None, :])
    rho /= rho.sum(axis=0)
    N = model.normalization_site_count()
    obs = {}
    e = (Es[:, None] * rho).sum(0)
    obs["Energy"] = e / N
    obs["SpecificHeat"] = ((Es[:, None] ** 2 * rho).sum(0) - e**2) / (Ts**2 * N)

    w2 = (np.abs(psi) ** 2)  # |<i|n>|^2

    def dmean(d):
        """thermal mean of an operator diagonal in the product basis"""
        Ann = d @ w2
        return (Ann[:, None] * rho).sum(0)

    for spec in model.get_opstring_estimators():
        diag = np.zeros(int(lif.cum[-1]))
        for i in range(1, model.lattice.site_count() + 1):
            sg = model.lattice.staggered_sign(spec.ordering_vector, spec.stagger_uc, i)
            loc = np.diag([model.magnetization_state(i, s) for s in range(1, lif.dims[i - 1] + 1)])
            diag += sg * lif.lift(i, loc).diagonal()
        diag /= N
        m2 = dmean(diag**2)
        m4 = dmean(diag**4)
        obs[spec.prefix + "Mag"] = dmean(diag)
        obs[spec.prefix + "Mag2"] = m2
        obs[spec.prefix + "Mag4"] = m4
        obs[spec.prefix + "AbsMag"] = dmean(np.abs(diag))
        obs[spec.prefix + "BinderRatio"] = m2**2 / m4
        Mnm = psi.conj().T @ (diag[:, None] * psi)
        chi = []
        for k, T in enumerate(Ts):
            dE = Es[None, :] - Es[:, None]  # E_m - E_n at [n, m]
            denom = np.where(np.isclose(Es[:, None], Es[None, :], atol=1e-6), 2 * T, dE)
            chi.append(np.sum(2 * rho[:, k][:, None] / denom * Mnm * Mnm.T).real)
        obs[spec.prefix + "MagChi"] = np.array(chi) * N
    return obs


def evaluables(est_prefixes, norm_sites):
    """Carlo evaluables of src/sse.jl:111-134 and magnetization_estimator.jl:236-258,
    as functions of the mean of the raw observables (dict name -> mean)."""
    f = {
        "Energy": lambda o: o["SignEnergy"] / o["Sign"],
        "SpecificHeat": lambda o: (o["SignOperatorCount2"] / o["Sign"] - o["SignOperatorCount"] ** 2 / o["Sign"] ** 2
                                   - o["SignOperatorCount"] / o["Sign"]) / norm_sites,
    }
    for p in est_prefixes:
        for name in ("Mag", "AbsMag", "Mag2", "Mag4", "MagChi"):
            f[p + name] = (lambda key: (lambda o: o[key] / o["Sign"]))("Sign" + p + name)

        def binder(o, p=p):
            s2, s4 = o["Sign" + p + "Mag2"], o["Sign" + p + "Mag4"]
            if s2 == 0 and s4 == 0:
                return 0.0
            return s2**2 / s4 / o["Sign"]

        f[p + "BinderRatio"] = binder
    return f


def jackknife(bins: dict, func):
    """Mean and jackknife error of ``func`` over bin means (dict name -> array of bin means)."""
    keys = list(bins)
    nb = len(bins[keys[0]])
    tot = {k: np.sum(bins[k]) for k in keys}
    full = func({k: tot[k] / nb for k in keys})
    loo = np.array([func({k: (tot[k] - bins[k][i]) / (nb - 1) for k in keys}) for i in range(nb)])
    err = np.sqrt((nb - 1) / nb * np.sum((loo - loo.mean()) ** 2))
    return full, err
