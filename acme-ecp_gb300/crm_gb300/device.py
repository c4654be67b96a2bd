"""Device-resident copies of the crm() arguments, for crm_run_device.

Each array is a torch CUDA tensor whose memory has the same Fortran layout
(column index fastest) as the host type it mirrors, so the C ABI receives
plain device pointers.  torch is used only as the device allocator here.
"""
import ctypes as C

import numpy as np

from . import crm_types as T


def _dev(a, torch, dtype=None):
    """A CUDA tensor holding array a in Fortran order."""
    a = np.asfortranarray(a)
    t = torch.from_numpy(np.ascontiguousarray(a.T)).to('cuda')
    return t


def _p(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


class DeviceCrmArrays:
    """crm_input / crm_state / crm_rad / crm_output / gcol on the device."""

    def __init__(self, cfg, cin, state, rad, desc, gcol):
        import torch
        self.torch = torch
        self.ld = desc.ld
        self.inp = {n: _dev(a, torch) for n, a in cin.arrays().items()}
        self.state = {n: _dev(a, torch) for n, a in state.arrays().items()}
        self.rad = {n: _dev(a, torch) for n, a in rad.arrays().items()}
        out = T.CrmOutput(desc.ld, cfg.crm_nx, cfg.crm_ny, cfg.crm_nz, cfg.plev)
        self.out = {n: _dev(a, torch) for n, a in out.arrays().items()}
        self.gcol = torch.tensor(np.asarray(gcol, dtype=np.int32), device='cuda')
        self.status = torch.zeros(desc.ncrms, dtype=torch.int32, device='cuda')
        self.status_ptr = self.status.data_ptr()
        self.c_in = T.CCrmInput(*[_p(self.inp[n]) for n in T.INPUT_FIELDS])
        self.c_state = T.CCrmState(*[_p(self.state[n]) for n in T.STATE_FIELDS])
        self.c_rad = T.CCrmRad(*[_p(self.rad[n]) for n in T.RAD_FIELDS])
        self.c_out = T.CCrmOutput()
        for i, (n, _) in enumerate(T.OUTPUT_FIELDS):
            self.c_out.field[i] = _p(self.out[n])
        self.c_desc = T.CCrmCallDesc(desc.lchnk, desc.ncrms, desc.ld, desc.dt_gl, desc.igstep,
                                     C.cast(C.c_void_p(self.gcol.data_ptr()), C.POINTER(C.c_int)))

    def reset_state(self, state):
        for n, a in state.arrays().items():
            self.state[n].copy_(self.torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)))

    def state_numpy(self, name):
        return self.state[name].cpu().numpy().T

    def out_numpy(self, name):
        return self.out[name].cpu().numpy().T

    def nbytes_state(self):
        return sum(t.numel() * t.element_size() for t in self.state.values())
