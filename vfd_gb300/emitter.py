"""Inflow emitter (the reference has none): particles enter through a disk, layer by layer.

A layer is the set of lattice points of spacing 2r (square lattice in the disk's plane)
within the disk of radius R. Each time the layer emitted last has travelled one spacing
along the inflow direction at the inflow speed, the next one is added through
DFSPHSimulation.Emit (vfd_emit) at the disk, shifted forward by the distance the flow has
covered past that spacing, so that layers stay evenly spaced whatever the time step.
"""
from __future__ import annotations

import numpy as np


def _basis(direction):
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    a = np.array([1.0, 0.0, 0.0]) if abs(d[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(d, a)
    u /= np.linalg.norm(u)
    return d, u, np.cross(d, u)


class InflowEmitter:
    def __init__(self, center, direction, radius: float, speed: float, particle_radius: float):
        self.center = np.asarray(center, np.float64)
        self.d, self.u, self.w = _basis(direction)
        self.radius, self.speed = float(radius), float(speed)
        self.spacing = 2.0 * float(particle_radius)
        k = int(np.floor(self.radius / self.spacing))
        ij = np.array([(i, j) for i in range(-k, k + 1) for j in range(-k, k + 1)], np.float64) * self.spacing
        self.disk = ij[np.sum(ij * ij, axis=1) <= self.radius * self.radius]
        self.travel = 0.0  # distance the last layer has moved since it was emitted
        self.emitted = 0
        self.layers = 0

    def layer(self, offset: float = 0.0):
        """Positions and velocities of one layer, `offset` along the inflow direction."""
        x = self.center + offset * self.d + self.disk[:, :1] * self.u + self.disk[:, 1:] * self.w
        v = np.tile(self.speed * self.d, (len(x), 1))
        return x.astype(np.float32), v.astype(np.float32)

    def advance(self, sim, dt: float) -> int:
        """Emits the layers due after `dt` more seconds of flow; returns the count added."""
        self.travel += self.speed * float(dt)
        added = 0
        while self.travel >= self.spacing:
            self.travel -= self.spacing
            x, v = self.layer(self.travel)
            sim.Emit(x, v)
            added += len(x)
            self.layers += 1
        self.emitted += added
        return added

    def run(self, sim, steps: int, on_step=None) -> dict:
        """`steps` steps of `sim`, emitting as the flow requires after each one."""
        st = {}
        for k in range(steps):
            st = sim.OnUpdate()
            self.advance(sim, st["TimeStepSize"])
            if on_step is not None:
                on_step(k, st)
        return st
