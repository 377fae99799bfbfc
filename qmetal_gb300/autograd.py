"""Adjoint differentiation as a torch.autograd.Function.

``energy(angles, template, hamiltonian, sim)`` returns E(angles) =
<psi(angles)|H|psi(angles)> as a 0-d float64 tensor whose backward pass is
the simulator's adjoint gradient (qm_energy_and_gradient: one forward pass,
a co-state lambda = H psi, and a backward sweep that takes Im<lambda|P|psi>
for every RX/RY/RZ and undoes both states). `angles` carries one entry per
parameterised gate of `template`, in circuit order, so any torch expression
that produces them (tied or scaled parameters, e.g. QAOA's RZ(2 gamma)) gets
its chain rule from autograd.

The GPU state lives behind the ctypes handle; torch only carries the angles
and the gradient (CPU float64).
"""
from __future__ import annotations

import torch

from . import Circuit, Hamiltonian, Simulator


class Template:
    """A gate stream whose parameterised gates take their angle from a vector."""

    def __init__(self, num_qubits, gates):
        self.num_qubits = int(num_qubits)
        self.gates = [(int(k), tuple(int(q) for q in qs), tuple(float(p) for p in ps))
                      for k, qs, ps in gates]
        self.param_index = [i for i, (_k, _q, ps) in enumerate(self.gates) if ps]

    @property
    def num_params(self):
        return len(self.param_index)

    def angles(self):
        return [self.gates[i][2][0] for i in self.param_index]

    def circuit(self, angles):
        a = [float(x) for x in angles]
        if len(a) != self.num_params:
            raise ValueError(f"expected {self.num_params} angles, got {len(a)}")
        c = Circuit(self.num_qubits)
        it = iter(a)
        for k, qs, ps in self.gates:
            c.add(k, qs, (next(it),) if ps else ())
        return c


def _ham(h):
    if isinstance(h, Hamiltonian):
        return h
    out = Hamiltonian()
    for c, x, y, z in h:
        out.add(c, x, y, z)
    return out


class AdjointEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, angles, template, hamiltonian, sim):
        c = template.circuit(angles.detach().cpu().double().tolist())
        e, g = sim.energy_and_gradient(c, hamiltonian)
        grad = torch.tensor([g[i] for i in template.param_index], dtype=torch.float64)
        ctx.save_for_backward(grad)
        return torch.tensor(e, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return grad_out * grad, None, None, None


def energy(angles: torch.Tensor, template: Template, hamiltonian, sim: Simulator | None = None):
    """Differentiable energy; the gradient comes from the adjoint sweep."""
    if sim is None:
        sim = Simulator(template.num_qubits)
    a = angles.to(torch.float64)
    if a.device.type != "cpu":
        a = a.cpu()
    return AdjointEnergy.apply(a, template, _ham(hamiltonian), sim)
