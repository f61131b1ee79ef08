"""Case files and the headless simulation loop over the library's C ABI.

Mirrors the reference's host classes with their method names, so a script
written against them reads the same:

* ``Input`` -- reference src/input.cpp (loadParameters, loadSolids and the
  getters/setters the simulation reads);
* ``SimulationD2Q9`` / ``SimulationD3Q19`` -- the constructors' initial state
  (reference src/simulation_d2q9.cu:55-390, src/simulation_d3q19.cu:50-289)
  and runLBM (src/simulation_d2q9.cu:423-560, src/simulation_d3q19.cu:321-436)
  driving the drop-in entry points, with a plain device buffer as the plot
  buffer instead of a mapped GL buffer;
* ``Output`` -- reference src/output.cpp (saveParVTK, saveVTK, getMLUPS).

One GPU: a case written for several devices runs as one device over the whole
width (the reference splits the width into device slabs joined by border
exchange; the lattice update is the same).
"""
import ctypes
import os
import time

import numpy as np

from . import abi
from .lattice import DeviceData, LBError, W2, W3, _lib, _ptr


def _check(rc, what):
    if rc != abi.LB_OK:
        raise LBError("%s failed (%d): %s" % (what, rc, _lib().lb_abi_last_error().decode()))


def _bytes(path):
    return os.fsencode(path)


class Input:
    """reference src/input.h: case parameters and the solid mask."""

    def __init__(self):
        self.p = abi.lb_case_params()
        self.p.max_dim = 1
        self.width = self.height = 0
        self.depth = 1
        self.solids = None          # uint8 (depth, height, width)

    # -- files -----------------------------------------------------------
    def loadParameters(self, fileName):
        """reference src/input.cpp:51-94; False when the file cannot be read."""
        rc = _lib().lb_case_load_parameters(_bytes(fileName), ctypes.byref(self.p))
        if rc == abi.LB_ERR_IO:
            return False
        _check(rc, "lb_case_load_parameters")
        if self.p.max_dim <= 1:
            self.depth = 1
        return True

    def loadSolids(self, fileName):
        """reference src/input.cpp:96-116: black pixels of a bitmap are solid."""
        L = _lib()
        w, h = ctypes.c_int(), ctypes.c_int()
        rc = L.lb_case_load_solids_bmp(_bytes(fileName), ctypes.byref(w), ctypes.byref(h),
                                       None, 0)
        if rc == abi.LB_ERR_IO:
            return False
        _check(rc, "lb_case_load_solids_bmp")
        mask = np.zeros(w.value * h.value, np.uint8)
        _check(L.lb_case_load_solids_bmp(_bytes(fileName), ctypes.byref(w), ctypes.byref(h),
                                         _ptr(mask), mask.nbytes), "lb_case_load_solids_bmp")
        self.width, self.height, self.depth = w.value, h.value, 1
        self.solids = mask.reshape(1, h.value, w.value)
        return True

    def loadSolidsSTL(self, fileName):
        """reference src/input.cpp:118-142: the solids of a 3-D case, voxelised
        on the GPU at maxDim voxels along the longest side (lb_voxelize)."""
        L = _lib()
        n = ctypes.c_int64()
        rc = L.lb_stl_read(_bytes(fileName), ctypes.byref(n), None, 0)
        if rc == abi.LB_ERR_IO:
            return False
        _check(rc, "lb_stl_read")
        tri = np.zeros(9 * n.value, np.float32)
        _check(L.lb_stl_read(_bytes(fileName), ctypes.byref(n), _ptr(tri), tri.size),
               "lb_stl_read")
        dims = (ctypes.c_int * 3)()
        _check(L.lb_voxelize(_ptr(tri), n.value, self.getMaxDim(), dims, None, 0, None),
               "lb_voxelize")
        mask = np.zeros(dims[0] * dims[1] * dims[2], np.uint8)
        _check(L.lb_voxelize(_ptr(tri), n.value, self.getMaxDim(), dims, _ptr(mask), mask.nbytes,
                             None), "lb_voxelize")
        self.width, self.height, self.depth = dims[0], dims[1], dims[2]
        self.solids = mask.reshape(dims[2], dims[1], dims[0])
        return True

    def setSolids(self, solids):
        """A solid mask from the caller: (height, width) or (depth, height,
        width)."""
        s = np.asarray(solids, np.uint8)
        if s.ndim == 2:
            s = s[None]
        self.depth, self.height, self.width = s.shape
        self.solids = np.ascontiguousarray(s)

    def loadFile(self, fileName):
        """reference src/mainwindow.cpp:237-265 without the widgets: the .dat
        file, then the .bmp of the same name for a 2-D case."""
        if not self.loadParameters(fileName):
            raise LBError("cannot read file %s" % fileName)
        if self.getMaxDim() > 1:
            stl = fileName[:-3] + "stl"
            if not self.loadSolidsSTL(stl):
                raise LBError("cannot read file %s" % stl)
            return self
        bmp = fileName[:-3] + "bmp"
        if not self.loadSolids(bmp):
            raise LBError("cannot read file %s" % bmp)
        return self

    # -- getters / setters (reference src/input.cpp:144-214) --------------
    def getWidth(self): return self.width
    def getHeight(self): return self.height
    def getLength(self): return self.depth
    def getMaxDim(self): return self.p.max_dim
    def getDeviceCount(self): return self.p.device_count
    def getUx(self): return self.p.ux
    def getUy(self): return self.p.uy
    def getUz(self): return self.p.uz
    def getRho(self): return self.p.rho
    def getViscosity(self): return self.p.viscosity
    def getTauInv(self): return self.p.tau_inv
    def getUpdateSteps(self): return self.p.update_steps
    def getExtFx(self): return self.p.ext_f[0]
    def getExtFy(self): return self.p.ext_f[1]
    def getExtFz(self): return self.p.ext_f[2]
    def getG(self): return self.p.G
    def getGads(self): return self.p.G_ads
    def getSolids(self): return self.solids
    def getMinU(self): return self.p.min_u
    def getMaxU(self): return self.p.max_u
    def getMinRho(self): return self.p.min_rho
    def getMaxRho(self): return self.p.max_rho

    def setUx(self, v): self.p.ux = v
    def setUy(self, v): self.p.uy = v
    def setUz(self, v): self.p.uz = v
    def setRho(self, v): self.p.rho = v
    def setUpdateSteps(self, v): self.p.update_steps = int(v)
    def setG(self, v): self.p.G = v
    def setGads(self, v): self.p.G_ads = v

    def setViscosity(self, v):
        """tau_inv = 1/(3 nu + 0.5) in double, stored as float
        (src/input.cpp:168-171)."""
        self.p.viscosity = v
        self.p.tau_inv = float(np.float32(1.0 / (3.0 * float(np.float32(v)) + 0.5)))

    def params_dict(self):
        p = self.p
        return dict(device_count=p.device_count, max_dim=p.max_dim, ux=p.ux, uy=p.uy, uz=p.uz,
                    rho=p.rho, viscosity=p.viscosity, update_steps=p.update_steps,
                    ext_f=list(p.ext_f), G=p.G, G_ads=p.G_ads, tau_inv=p.tau_inv,
                    min_u=p.min_u, max_u=p.max_u, min_rho=p.min_rho, max_rho=p.max_rho)


class Output:
    """reference src/output.cpp: VTK files and the MLUPS figure."""

    def __init__(self, inp, device_count=1):
        self.deviceCount = device_count
        self.width = inp.getWidth() // device_count
        self.height = inp.getHeight()
        self.length = inp.getLength()
        self.updateSteps = inp.getUpdateSteps()
        self.vtkId = 0
        self.lbmTime = 0.0

    def saveParVTK(self, directory=""):
        _check(_lib().lb_vtk_save_parallel(_bytes(directory), self.vtkId, self.deviceCount,
                                           self.width, self.height, self.length),
               "lb_vtk_save_parallel")

    def saveVTK(self, deviceID, rho, ux, uy, uz=None, directory=""):
        rho, ux, uy = (np.ascontiguousarray(a, np.float32) for a in (rho, ux, uy))
        uzp = None if uz is None else _ptr(np.ascontiguousarray(uz, np.float32))
        _check(_lib().lb_vtk_save(_bytes(directory), self.vtkId, deviceID, self.width,
                                  self.height, self.length, _ptr(rho), _ptr(ux), _ptr(uy), uzp),
               "lb_vtk_save")
        if deviceID == self.deviceCount - 1:
            self.vtkId += 1

    def getMLUPS(self):
        """1e-6 * updateSteps * nodes / lbmTime (src/output.cpp:172)."""
        return 1e-6 * self.updateSteps * self.width * self.height * self.length / self.lbmTime


class _Simulation:
    Q = 0

    def __init__(self, inp):
        if inp.getSolids() is None:
            raise LBError("the case has no solid mask")
        self.input = inp
        self.width, self.height, self.depth = inp.getWidth(), inp.getHeight(), inp.getLength()
        self.size = self.width * self.height * self.depth
        self.output = Output(inp)
        self.steps = 0
        self.cursor = [self.width // 2, self.height // 2, self.depth // 2]
        self.valueCur = np.zeros(4, np.float32)
        self.init = self._initial_state()
        self.data = DeviceData(self.Q, self.width, self.height, self.depth)
        d = self.data
        d.upload(self.init["f"])
        d.set_solid(inp.getSolids().reshape(-1), self.init["solid_bound"])
        for name in self.MOMENTS:
            d.h2d(getattr(d.s, name), self.init[name])

    def close(self):
        if getattr(self, "data", None) is not None:
            self.data.close()
            self.data = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def getOutput(self):
        return self.output

    def getSteps(self):
        return self.steps

    def populations(self):
        return self.data.download()

    def field(self, name):
        return self.data.field(name)

    def runLBM(self, updateSteps=None):
        """updateSteps times: streaming, collision into the plot buffer,
        read_value at the cursor and its 16-byte copy to the host."""
        n = self.input.getUpdateSteps() if updateSteps is None else int(updateSteps)
        L = _lib()
        self.output.updateSteps = n
        L.lb_device_synchronize()
        L.lb_abi_clear_error()  # report only what this run's entry points record
        t0 = time.perf_counter()
        for _ in range(n):
            self._step(L)
            self.steps += 1
        L.lb_device_synchronize()
        self.output.lbmTime = time.perf_counter() - t0
        err = L.lb_abi_last_error()
        if err:
            raise LBError(err.decode())

    def saveVTK(self, directory=""):
        """reference src/simulation_d2q9.cu:562-580 / _d3q19.cu:438-456."""
        self.output.saveParVTK(directory)
        uz = self.field("uz") if self.Q == 19 else None
        self.output.saveVTK(0, self.field("rho"), self.field("ux"), self.field("uy"), uz,
                            directory)


class SimulationD2Q9(_Simulation):
    Q = 9
    MOMENTS = ("ux", "uy", "rho", "psi", "ueq_x", "ueq_y")

    def _initial_state(self):
        N = self.size
        out = dict(f=np.zeros((9, N), np.float32), solid_bound=np.zeros(N, np.uint8))
        for k in self.MOMENTS:
            out[k] = np.zeros(N, np.float32)
        solids = np.ascontiguousarray(self.input.getSolids().reshape(-1), np.uint8)
        _check(_lib().lb_case_init_d2q9(
            ctypes.byref(self.input.p), self.width, self.height, _ptr(solids), _ptr(out["f"]),
            _ptr(out["ux"]), _ptr(out["uy"]), _ptr(out["rho"]), _ptr(out["psi"]),
            _ptr(out["ueq_x"]), _ptr(out["ueq_y"]), _ptr(out["solid_bound"])),
            "lb_case_init_d2q9")
        return out

    def _step(self, L):
        i, d = self.input, self.data
        F = ctypes.c_float
        g, b = abi.dim3(self.width // 32 or 1, self.height // 4 or 1, 1), abi.dim3(32, 4, 1)
        L.streaming_d2q9(d.ptr(), g, b)
        L.collision_d2q9(ctypes.c_void_p(d.plot), d.ptr(), F(W2[0]), F(W2[1]), F(W2[2]),
                         F(i.getTauInv()), F(i.getUx()), F(i.getUy()), F(i.getRho()),
                         F(i.getMinU()), F(i.getMaxU()), F(i.getMinRho()), F(i.getMaxRho()),
                         g, b, F(i.getExtFx()), F(i.getExtFy()), F(i.getG()), F(i.getGads()))
        x, y, z = self.cursor
        L.read_value_2d(ctypes.c_void_p(d.plot), d.ptr(), x, y, z)
        L.lb_memcpy_d2h(_ptr(self.valueCur), ctypes.c_void_p(d.s.valueCur), 16)


class SimulationD3Q19(_Simulation):
    Q = 19
    MOMENTS = ("ux", "uy", "uz", "rho")

    def _initial_state(self):
        N = self.size
        out = dict(f=np.zeros((19, N), np.float32), solid_bound=np.zeros(N, np.uint8))
        for k in self.MOMENTS:
            out[k] = np.zeros(N, np.float32)
        solids = np.ascontiguousarray(self.input.getSolids().reshape(-1), np.uint8)
        _check(_lib().lb_case_init_d3q19(
            ctypes.byref(self.input.p), self.width, self.height, self.depth, _ptr(solids),
            _ptr(out["f"]), _ptr(out["ux"]), _ptr(out["uy"]), _ptr(out["uz"]), _ptr(out["rho"]),
            _ptr(out["solid_bound"])), "lb_case_init_d3q19")
        return out

    def _step(self, L):
        i, d = self.input, self.data
        F = ctypes.c_float
        g, b = abi.dim3(self.width // 32 or 1, self.height // 4 or 1, self.depth), \
            abi.dim3(32, 4, 1)
        L.streaming_d3q19(d.ptr(), g, b)
        L.collision_d3q19(ctypes.c_void_p(d.plot), d.ptr(), F(W3[0]), F(W3[1]), F(W3[2]),
                          F(i.getTauInv()), F(i.getUx()), F(i.getUy()), F(i.getUz()),
                          F(i.getRho()), F(i.getMinU()), F(i.getMaxU()), F(i.getMinRho()),
                          F(i.getMaxRho()), g, b)
        x, y, z = self.cursor
        L.read_value_3d(ctypes.c_void_p(d.plot), d.ptr(), x, y, z)
        L.lb_memcpy_d2h(_ptr(self.valueCur), ctypes.c_void_p(d.s.valueCur), 16)


def load_case(fileName):
    """Input.loadFile plus the matching simulation (reference
    src/mainwindow.cpp:267-268: D3Q19 when the case has depth)."""
    inp = Input().loadFile(fileName)
    return SimulationD3Q19(inp) if inp.getLength() > 1 else SimulationD2Q9(inp)
