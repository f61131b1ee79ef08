"""The oracle's emulation of the library's population storage for the GPU
parity tests: FP32 keeps f itself; 16-bit storage keeps the deviations
d_k = f_k - w_k rho_ref, stepped with the deviation arithmetic and narrowed
and widened on every store (what the step kernels do)."""
import numpy as np


class Emulated:
    def __init__(self, oracle, f0, storage, rho_ref):
        self.o, self.storage = oracle, storage
        self.wr = oracle.storage_offsets(19, rho_ref)
        f0 = np.ascontiguousarray(f0, np.float32)
        self.state = f0.copy() if storage == 0 else oracle.to_dev(f0, self.wr, storage)

    def step(self, flags, corr, W, H, D, mom, w, tau_inv, F=(0, 0, 0), G=0.0, psi=None,
             psi_form=None):
        o = self.o
        psi_form = o.PSI_EXP1 if psi_form is None else psi_form
        o.d3q19_stream_native(self.state, flags, corr, W, H, D)
        if self.storage == 0:
            o.d3q19_collide_native(self.state, flags, mom, W, H, D, *w, tau_inv, F, G=G, psi=psi,
                                   psi_form=psi_form)
        else:
            o.d3q19_collide_native_dev(self.state, flags, mom, W, H, D, *w, tau_inv, self.wr, F,
                                       G=G, psi=psi, psi_form=psi_form)
            o.quantize(self.state, self.storage)

    def populations(self):
        """Float populations, as lb_get_populations returns them."""
        if self.storage == 0:
            return self.state
        return self.o.from_dev(self.state, self.wr)
