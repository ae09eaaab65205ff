"""Modified Broyden mixing of the induced potential (mix_potential_c,
phys/coul/src/mix_pot_c.f90:25-189), restated on the host.

The reference mixes the complex induced potential dvscfin of one
perturbation (all frequencies) between the iterations of the self-consistent
screening loop (solve_linter.f90:376-458, 560-575): with vout the Hartree
potential of the response density, it keeps the differences of the last
n_iter residuals (df) and inputs (dv), each pair normalised by |df|, builds
beta = (w0^2 + w_i^2 on the diagonal, w_i w_j <df_j|df_i> off it)^-1
(ZHETRF/ZHETRI; w_i = 1, w0 = 0.01) and returns
    vin + alpha (vout - vin) - sum_i w_i gamma_i (alpha df_i + dv_i),
    gamma_i = sum_j beta_ji w_j <df_j|vout - vin>.
Convergence: dr2 = (|vout - vin| / ndim)^2 < tr2.  The vectors here are the
coefficients of the potential on the perturbation set (a few thousand
numbers), so the host does this work, as the reference does.
"""
from __future__ import annotations

import numpy as np


class BroydenMixer:
    """State of mix_potential_c for one perturbation (its saved df/dv history)."""

    W0 = 0.01
    MAXTER = 8

    def __init__(self, n_iter=4):
        self.n_iter = min(int(n_iter), self.MAXTER)
        self.df = []
        self.dv = []
        self.iter = 0
        self._last_vout = None
        self._last_vin = None

    def mix(self, vout, vin, alphamix, tr2):
        """One call of mix_potential_c: returns (vin_new, dr2, conv); vout is the
        new output potential, vin the input potential of this iteration."""
        self.iter += 1
        vout = np.asarray(vout, dtype=np.complex128).ravel()
        vin = np.asarray(vin, dtype=np.complex128).ravel()
        res = vout - vin
        ndim = res.size
        dr2 = (np.linalg.norm(res) / ndim) ** 2
        conv = dr2 < tr2
        if conv:
            self.df, self.dv = [], []
            return vin.copy(), dr2, True
        if self.iter > 1:
            # differences to the previous call's residual and input, normalised by |df|
            df = res - self._last_vout
            dv = vin - self._last_vin
            nrm = np.linalg.norm(df)
            self.df.append(df / nrm)
            self.dv.append(dv / nrm)
            if len(self.df) > self.n_iter:
                self.df.pop(0)
                self.dv.pop(0)
        used = len(self.df)
        new = vin + alphamix * res
        if used:
            F = np.array(self.df)                       # (used, ndim)
            beta = F.conj() @ F.T                        # <df_i|df_j>
            beta = beta.T.copy()                         # beta[i, j] = <df_j|df_i>
            beta[np.diag_indices(used)] = self.W0 ** 2 + 1.0
            binv = np.linalg.inv(beta)
            work = F.conj() @ res                        # <df_i|vout - vin>
            gamma = binv.T @ work                        # gamma_i = sum_j beta_ji work_j
            for i in range(used):
                new = new - gamma[i] * (alphamix * self.df[i] + self.dv[i])
        self._last_vout = res
        self._last_vin = vin.copy()
        return new, dr2, False
