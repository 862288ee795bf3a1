"""CPU restatement of multiRegionFoam's partitioned Dirichlet-Neumann
interface coupling (test infrastructure only: tests import it as the
checker of the GPU kernels in multiregionfoam_gb300/csrc/dn.cu).

Each function cites the reference file:line it follows (paths within the
multiRegionFoam repository).  Scalar fields; patch A carries the jump
(Dirichlet) condition, patch B the flux (Neumann) condition.

  jump update   genericRegionCoupledJumpFvPatchField.C:164-217 with
                regionCoupledTemperatureJump::valueJump (regionCoupled
                TemperatureJump.C:83-104): value_A = nbr + (K - 1) nbr = K nbr,
                nbr = GGI-interpolated patch value of B, then relaxed
  flux update   genericRegionCoupledFluxFvPatchField.C:172-239 with
                regionCoupledHeatFlux::fluxJump = 0 (regionCoupledHeatFlux.C:
                83-86): grad_B = (-interp(k_A snGrad_A) + jump) / k_B, relaxed
  residuals     rawResidual / normResidual, Jump .C:244-332 and Flux
                .C:241-409: sqrt(sum raw^2) / max(min(|own|, |nbr + jump|), SMALL)
  relaxation    accelerationModel::updateResiual (accelerationModel.C:78-85),
                fixedRelaxation::relax (fixedRelaxation.C:76-101),
                aitkenRelaxation::relax / updateAitkenFactor
                (aitkenRelaxation.C:74-100, aitkenRelaxationTemplates.C:105-165),
                IQNILS::relax / updateVW (IQNILS.C:96-201) and updateIQNILS
                (IQNILSTemplates.C:44-133): modified Gram-Schmidt QR of the
                residual-difference columns, least squares, back-substitution
                with near-zero columns dropped
  criteria      dnaControl::criteriaSatisfied (dnaControl.C:582-635): no
                check on the first coupling iteration; converged when every
                max residual is <= its limit
Patch values of a fixedValue / fixedGradient patch and snGrad follow foam:
snGrad = deltaCoeffs (patch - internal) on a fixed-value patch, and a
fixed-gradient patch's value is internal + gradient / deltaCoeffs.
"""
from __future__ import annotations

import numpy as np

SMALL = 1e-15   # foam's SMALL (double precision)


def gpu_sum(v, threads=1024):
    """The device's fixed-order sum over one CTA of `threads` threads: thread
    t adds elements t, t + threads, ... in order, then a halving tree."""
    v = np.asarray(v, dtype=np.float64)
    part = np.zeros(threads)
    for start in range(0, len(v), threads):
        c = v[start:start + threads]
        part[:len(c)] = part[:len(c)] + c
    s = threads // 2
    while s:
        part[:s] = part[:s] + part[s:2 * s]
        s //= 2
    return float(part[0])


def seq_sum(v):
    """foam's sum of a field: element after element."""
    acc = 0.0
    for x in np.asarray(v, dtype=np.float64):
        acc += x
    return acc


IQN_MODES = 32   # columns kept per field; the oldest is dropped beyond this


class Relaxation:
    """fixedRelaxation (model 0), aitkenRelaxation (model 1) or IQNILS
    (model 2, couplingReuse `reuse`) of one field.  IQN-ILS sums in foam's
    element order, or with order="gpu" in the device's CTA order."""

    def __init__(self, model: int, relax: float, init_field, reuse: int = 0, order: str = "foam"):
        self.model = model
        self.init_relax = relax
        self.aitken = relax            # aitkenRelax_ starts at the initial factor
        self.corr = 1
        self.prev = np.array(init_field, dtype=np.float64)
        self.res = np.zeros_like(self.prev)
        self.prev_res = np.zeros_like(self.prev)
        # IQN-ILS history: columns oldest first, with their time indices
        self.reuse = reuse
        self.time_index = 0
        self.V, self.W, self.T = [], [], []
        self.fld_ref = self.res_ref = None
        self.sum = gpu_sum if order == "gpu" else seq_sum

    def new_time_step(self):
        self.corr = 1
        self.time_index += 1

    def _update_vw(self, cur):
        """IQNILS::updateVW (IQNILS.C:142-201)."""
        if self.corr == 1:
            while self.T and self.time_index - self.reuse > self.T[0]:
                del self.V[0], self.W[0], self.T[0]
        elif self.corr == 2:
            self.fld_ref = cur.copy()
            self.res_ref = self.res.copy()
        else:
            if len(self.T) == IQN_MODES:
                del self.V[0], self.W[0], self.T[0]
            self.V.append(self.res - self.res_ref)
            self.W.append(cur - self.fld_ref)
            self.T.append(self.time_index)

    def _update_iqnils(self, cur):
        """IQNILS<scalar>::updateIQNILS (IQNILSTemplates.C:44-133)."""
        cols = len(self.V)
        R = np.zeros((cols, cols))
        Cv = np.zeros(cols)
        Q = [self.V[cols - 1 - i].copy() for i in range(cols)]
        for i in range(cols):
            R[i, i] = np.sqrt(self.sum(Q[i] * Q[i]))
            Q[i] = Q[i] / R[i, i]
            for j in range(i + 1, cols):
                R[i, j] = self.sum(Q[i] * Q[j])
                Q[j] = Q[j] - R[i, j] * Q[i]
            Cv[i] = self.sum(Q[i] * (-self.res))
        colsum = []
        for j in range(cols):
            cs = 0.0
            for i in range(j + 1):
                cs += abs(R[i, j])
            colsum.append(cs)
        eps = 1.0e-10 * max(colsum)
        for i in range(cols):
            if abs(R[i, i]) > eps:
                for j in range(i + 1, cols):
                    R[i, j] = R[i, j] / R[i, i]
                Cv[i] = Cv[i] / R[i, i]
                R[i, i] = 1.0
        for j in range(cols - 1, -1, -1):
            if abs(R[j, j]) > eps:
                for i in range(j):
                    Cv[i] = Cv[i] - Cv[j] * R[i, j]
            else:
                Cv[j] = 0.0
        out = cur.copy()
        for i in range(cols):
            out = out + self.W[i] * Cv[cols - 1 - i]
        return out

    def relax(self, cur):
        cur = np.asarray(cur, dtype=np.float64)
        self.prev_res = self.res
        self.res = cur - self.prev
        if self.model == 2:
            self._update_vw(cur)
            if len(self.T) > 1:
                out = self._update_iqnils(cur)
            else:
                out = self.prev + self.init_relax * self.res
            self.prev = out
            self.corr += 1
            return out
        if self.model == 1:
            if self.corr < 3:
                self.aitken = self.init_relax if self.aitken < self.init_relax else self.aitken
            else:
                d = self.res - self.prev_res
                a = -self.aitken * (np.sum(self.prev_res * d) / (np.sum(d * d) + SMALL))
                a = abs(a)
                if a > 1.0:
                    a = 1.0
                elif a < SMALL:
                    a = self.init_relax
                self.aitken = a
            w = self.aitken
        else:
            w = self.init_relax
        out = self.prev + w * self.res
        self.prev = out
        self.corr += 1
        return out


class DnInterface:
    """One conformal or GGI interface: A (jump / Dirichlet), B (flux / Neumann).

    a_from_b / b_from_a: (ptr, addr, w) GGI CSR giving each face of one patch
    from the faces of the other.  fc_*: faceCells, delta_*: deltaCoeffs, k_*:
    face diffusivity, area_*: face areas.
    """

    def __init__(self, a_from_b, b_from_a, fc_a, delta_a, k_a, area_a, fc_b, delta_b, k_b, area_b,
                 K=1.0, flux_jump=0.0, model=1, relax=0.75, value_a0=None, grad_b0=None, reuse=0, order="foam",
                 model_b=None, relax_b=None):
        """model / relax / reuse: each patch's accelerationModel (accType,
        relax, couplingReuse); B takes A's unless model_b / relax_b say
        otherwise (a patch without accType is fixed with relax 1)."""
        self.a_from_b, self.b_from_a = a_from_b, b_from_a
        self.fc_a, self.delta_a, self.k_a, self.area_a = fc_a, delta_a, k_a, area_a
        self.fc_b, self.delta_b, self.k_b, self.area_b = fc_b, delta_b, k_b, area_b
        self.K, self.flux_jump = K, flux_jump
        self.value_a = np.array(value_a0, dtype=np.float64)
        self.grad_b = np.array(grad_b0, dtype=np.float64)
        self.relax_a = Relaxation(model, relax, self.value_a, reuse, order)
        self.relax_b = Relaxation(model if model_b is None else model_b, relax if relax_b is None else relax_b,
                                  self.grad_b, reuse, order)

    def new_time_step(self):
        self.relax_a.new_time_step()
        self.relax_b.new_time_step()

    @staticmethod
    def _interp(csr, src):
        ptr, addr, w = csr
        out = np.zeros(len(ptr) - 1)
        for i in range(len(ptr) - 1):
            out[i] = np.dot(w[ptr[i]:ptr[i + 1]], src[addr[ptr[i]:ptr[i + 1]]])
        return out

    def face_b(self, t_b):
        return t_b[self.fc_b] + self.grad_b / self.delta_b

    def flux_a(self, t_a):
        return self.k_a * self.delta_a * (self.value_a - t_a[self.fc_a])

    def update_a(self, t_b):
        nbr = self._interp(self.a_from_b, self.face_b(t_b))
        self.value_a = self.relax_a.relax(nbr + (self.K - 1.0) * nbr)
        return self.value_a

    def update_b(self, t_a):
        f = -self._interp(self.b_from_a, self.flux_a(t_a)) + self.flux_jump
        self.grad_b = self.relax_b.relax(f / self.k_b)
        return self.grad_b

    def rhs_a(self, b0):
        b = np.array(b0, dtype=np.float64)
        np.add.at(b, self.fc_a, self.k_a * self.area_a * self.delta_a * self.value_a)
        return b

    def rhs_b(self, b0):
        b = np.array(b0, dtype=np.float64)
        np.add.at(b, self.fc_b, self.k_b * self.area_b * self.grad_b)
        return b

    def residuals(self, t_a, t_b):
        """(jump normResidual on A, flux normResidual on B)."""
        nbr = self._interp(self.a_from_b, self.face_b(t_b))
        jump = (self.K - 1.0) * nbr
        raw = np.abs((self.value_a - nbr) - jump)
        nj = max(min(np.sqrt(np.sum(self.value_a ** 2)), np.sqrt(np.sum((nbr + jump) ** 2))), SMALL)
        fnbr = self._interp(self.b_from_a, self.flux_a(t_a))
        fown = self.grad_b * self.k_b
        rawf = np.abs((fown + fnbr) - self.flux_jump)
        nf = max(min(np.sqrt(np.sum(fown ** 2)), np.sqrt(np.sum((-fnbr + self.flux_jump) ** 2))), SMALL)
        return np.sqrt(np.sum(raw ** 2)) / nj, np.sqrt(np.sum(rawf ** 2)) / nf


def criteria_satisfied(corr: int, jump_res: float, flux_res: float, max_jump: float, max_flux: float) -> bool:
    """dnaControl::criteriaSatisfied for one field and interface."""
    if corr == 1:
        return False
    return jump_res <= max_jump and flux_res <= max_flux
