"""The learned return map: a 7 -> 64 -> 64 -> 64 -> 3 SiLU MLP with BF16 weights on
the tensor cores, trained on the GPU by libaep.so's own forward, backward and Adam
kernels from (trial, projected) pairs that the exact return mapping produces
(aep_set_harvest).  Device buffers are torch tensors (plumbing only); every
computation runs in libaep.so.

Record layout (8 float32): [ln s0, ln s1, ln s2 (trial, sorted descending), q,
material, d0, d1, d2], d = ln s_projected - ln s_trial; cloth element records
(material 2): [r13, r23, r33 - 1, cap ratio, 2, change of (r13, r23, r33)].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import AepError

NUM_PARAMS = capi.AEP_MLP_NUM_PARAMS
LN_SCALE = 50.0
# packed parameter blocks (W^T blocks are [out][in], row-major)
LAYOUT = [("w1t", (64, 16)), ("w2t", (64, 64)), ("w3t", (64, 64)), ("w4t", (8, 64)),
          ("b1", (64,)), ("b2", (64,)), ("b3", (64,)), ("b4", (8,))]


def unpack(p: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shape in LAYOUT:
        k = int(np.prod(shape))
        out[name] = p[off:off + k].reshape(shape)
        off += k
    assert off == NUM_PARAMS
    return out


class ReturnMapMLP:
    def __init__(self, seed: int = 0):
        self._lib = capi.load()
        self.handle = C.c_void_p()
        st = self._lib.aep_mlp_create(int(seed), C.byref(self.handle))
        if st != capi.AEP_OK:
            raise AepError(st, "aep_mlp_create")

    def _check(self, st):
        if st != capi.AEP_OK:
            raise AepError(st, self._lib.aep_mlp_last_error(self.handle).decode())

    def close(self):
        if self.handle:
            self._lib.aep_mlp_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        p = np.empty(NUM_PARAMS, np.float32)
        self._check(self._lib.aep_mlp_get_params(self.handle, p.ctypes.data_as(C.POINTER(C.c_float)), NUM_PARAMS))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self._lib.aep_mlp_set_params(self.handle, p.ctypes.data_as(C.POINTER(C.c_float)), NUM_PARAMS))

    def gradient(self, records_ptr: int, n: int) -> tuple[np.ndarray, float]:
        g = np.empty(NUM_PARAMS, np.float32)
        loss = C.c_double()
        self._check(self._lib.aep_mlp_gradient(self.handle, C.c_void_p(records_ptr), int(n),
                                               g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def train(self, records_ptr: int, n: int, steps: int, batch: int = 8192, lr: float = 2e-3,
              lr_final: float = 2e-5, stream_ptr: int = 0) -> float:
        loss = C.c_double()
        self._check(self._lib.aep_mlp_train(self.handle, C.c_void_p(records_ptr), int(n), int(steps), int(batch),
                                            float(lr), float(lr_final), C.byref(loss), C.c_void_p(stream_ptr)))
        return loss.value

    def forward(self, records_ptr: int, n: int, out_ptr: int, stream_ptr: int = 0, step_form: bool = False):
        """Predicted corrections of n device records; step_form: with the SiLU of the
        step's learned return map (aep_mlp_forward_step_form)."""
        fn = self._lib.aep_mlp_forward_step_form if step_form else self._lib.aep_mlp_forward
        self._check(fn(self.handle, C.c_void_p(records_ptr), int(n), C.c_void_p(out_ptr), C.c_void_p(stream_ptr)))


def canonical_order(recs):
    """The records sorted lexicographically by their 32-bit patterns: the kernels
    append records in whatever order their atomics run, so this fixes one order
    for a set of records (and with it the batches training draws)."""
    import torch

    bits = recs.view(torch.int32)
    order = torch.arange(len(recs), device=recs.device)
    for c in reversed(range(recs.shape[1])):  # least significant column first, stable sorts
        order = order[torch.sort(bits[order, c], stable=True).indices]
    return recs[order]


def harvest_records(scene, steps: int, capacity: int, stride: int = 1, warm_steps: int = 0, seed: int = 0):
    """Run the exact (plain) step on `scene` and return a torch CUDA tensor of at most
    `capacity` harvested records [count, 8], the same records on every run: the buffer
    holds every record the steps can produce (one per particle slot of stride and step,
    one per cloth element and step), the records are put in canonical order and, when
    there are more than `capacity`, a seeded uniform sample of them over all steps is
    kept."""
    import torch

    from .solver import HybridSolver

    n_items = scene.num_items()
    n_elem = len(scene.mesh.faces) if scene.mesh is not None else 0
    room = steps * (-(-n_items // stride) + n_elem)
    buf = torch.empty((room, 8), dtype=torch.float32, device="cuda")
    s = HybridSolver(scene.particles, scene.grid, scene.params)
    if scene.mesh is not None:
        s.set_lagrangian_mesh(scene.mesh)
    s.set_level_set(scene.levelset)
    s.init_volumes()
    for _ in range(warm_steps):
        s.step(scene.dt)
    s.set_harvest(buf.data_ptr(), room, stride)
    for _ in range(steps):
        s.step(scene.dt)
    cnt = s.harvest_count()
    s.set_harvest(None)
    s.close()
    if cnt >= room:
        raise RuntimeError(f"harvest buffer of {room} records filled")
    recs = canonical_order(buf[:cnt])
    del buf
    if cnt > capacity:
        keep = torch.randperm(cnt, generator=torch.Generator().manual_seed(seed))[:capacity]
        recs = recs[torch.sort(keep).values.to(recs.device)]
    return recs.contiguous()
