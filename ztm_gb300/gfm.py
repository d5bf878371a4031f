"""Host-side mirror of ZTM's gravity call surface over the C ABI.

The reference's gravity path is the block of FM::FM at TFM.cpp:83-99: it
takes the fine-grid density perturbation `drho` (built at TFM.cpp:85-89), the
station heights `surf = topo + sea` and returns the field `G` (mGal) on the
di x dj grid, either through the GFM process (TFM.cpp:90-94) or the CPU
lambda (TFM.cpp:95-99).  `GravityContext.pointmass` is that call.  The prism,
interface, adjoint and batched calls extend it with the closed-form model.

Arrays may be numpy arrays (host memory: the library copies in and out) or
CUDA torch tensors (device memory: used in place, the call is asynchronous on
the context's stream).  Every call goes through libztmgrav.so; there is no
CPU fallback, and a non-zero status raises GravityError.
"""
import ctypes

import numpy as np

from . import _lib

PRECISIONS = {"fp64": _lib.PREC_FP64, "fp32": _lib.PREC_FP32, "mixed": _lib.PREC_MIXED}
DEFAULT_G = 6.67e-11  # the constant behind the 66.7 mGal factor of TFM.cpp:98
AUTOTUNE = 2  # ZTM_FLAG_AUTOTUNE


class GravityError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ztm status %d: %s" % (code, msg))
        self.code = code


def _is_torch_cuda(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


class _Args:
    """Collects array arguments of one call; all host or all device.

    Device tensors are used by kernels queued on the context's stream after
    the call returns.  GravityContext._run makes PyTorch's current stream
    wait for that work, so memory that PyTorch frees after the call and
    hands to a later tensor is only touched by work ordered after the
    library's kernels."""

    def __init__(self, gctx=None):
        self.device = None
        self.keep = []
        self.gctx = gctx

    def _kind(self, dev):
        if self.device is None:
            self.device = dev
        elif self.device != dev:
            raise ValueError("mix of host and device arrays in one call")

    def arr(self, x, n=None, dtype=np.float64, name="array"):
        if x is None:
            return None
        if _is_torch_cuda(x):
            import torch
            want = torch.float64 if dtype == np.float64 else torch.int32
            if x.dtype != want:
                raise TypeError("%s must be %s" % (name, want))
            if not x.is_contiguous():
                raise ValueError("%s must be contiguous" % name)
            if n is not None and x.numel() != n:
                raise ValueError("%s has %d elements, expected %d" % (name, x.numel(), n))
            self._kind(True)
            self.keep.append(x)
            return ctypes.c_void_p(x.data_ptr())
        a = np.ascontiguousarray(x, dtype=dtype)
        if n is not None and a.size != n:
            raise ValueError("%s has %d elements, expected %d" % (name, a.size, n))
        self._kind(False)
        self.keep.append(a)
        return a.ctypes.data_as(ctypes.c_void_p)

    def out(self, n, like=None):
        if self.device:
            import torch
            t = torch.empty(n, dtype=torch.float64, device=like.device if like is not None else "cuda")
            self.keep.append(t)
            return t, ctypes.c_void_p(t.data_ptr())
        a = np.empty(n, dtype=np.float64)
        self.keep.append(a)
        return a, a.ctypes.data_as(ctypes.c_void_p)

    def scalar(self, like=None):
        """A one-value output: a ctypes double (host) or a 1-element tensor
        (device); returns (holder, pointer)."""
        if self.device:
            import torch
            t = torch.zeros(1, dtype=torch.float64, device=like.device if like is not None else "cuda")
            self.keep.append(t)
            return t, ctypes.c_void_p(t.data_ptr())
        v = ctypes.c_double(0.0)
        self.keep.append(v)
        return v, ctypes.cast(ctypes.pointer(v), ctypes.c_void_p)

    @staticmethod
    def value(holder):
        return holder if not isinstance(holder, ctypes.c_double) else holder.value

    @property
    def flags(self):
        return _lib.FLAG_DEVICE_PTRS if self.device else 0


def make_grid(di, dj, dk, fh=1, fv=2, bfr=10, threshold=0.001, scale=1.0):
    """Reference grid (defaults: GFM_GPU.cu:24 for fh, fv, bfr)."""
    return _lib.Grid(di, dj, dk, fh, fv, bfr, threshold, scale)


def make_mesh(nx, ny, nz, dx, dy, dz, x0=0.0, y0=0.0, z_top=0.0):
    return _lib.Mesh(nx, ny, nz, x0, y0, z_top, dx, dy, dz)


def make_imesh(nx, ny, dx, dy, z_base, x0=0.0, y0=0.0):
    return _lib.IMesh(nx, ny, x0, y0, dx, dy, z_base)


def _opts(precision, flags, G, near_q, tile=0, chunk=0):
    if isinstance(precision, str):
        precision = PRECISIONS[precision]
    return _lib.Opts(precision, flags, G or 0.0, near_q or 0.0, tile, chunk)


class GravityContext:
    """One CUDA device, one stream, one grow-only workspace."""

    def __init__(self, device=0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self._lib.ztm_ctx_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise GravityError(rc, "context creation failed on device %d" % device)
        self._h = h
        self.device = device
        self._tstream = None

    # -- lifetime ------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.ztm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            msg = self._lib.ztm_last_error(self._h)
            raise GravityError(rc, msg.decode() if msg else "")

    def _run(self, a, fn, *args):
        """Call an entry point.  With device tensors, order the library's
        stream after PyTorch's current stream (inputs written there are
        complete) and PyTorch's after the library's (results are visible
        to later torch work); the host is not blocked."""
        if not a.device:
            self._check(fn(*args))
            return
        import torch
        ts = self._torch_stream()
        cur = torch.cuda.current_stream(self.device)
        if cur.cuda_stream != ts.cuda_stream:
            ts.wait_stream(cur)
        self._check(fn(*args))
        if cur.cuda_stream != ts.cuda_stream:
            cur.wait_stream(ts)

    @property
    def stream(self):
        return self._lib.ztm_ctx_stream(self._h)

    def set_stream(self, stream_ptr):
        self._check(self._lib.ztm_ctx_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))
        self._tstream = None

    def _torch_stream(self):
        """The context's stream as a torch stream object (for record_stream)."""
        if self._tstream is None:
            import torch
            self._tstream = torch.cuda.ExternalStream(self.stream, device=self.device)
        return self._tstream

    def launches(self):
        return int(self._lib.ztm_ctx_launches(self._h))

    def sync(self):
        self._check(self._lib.ztm_ctx_sync(self._h))

    # -- tracing ----------------------------------------------------------
    def profile(self, enable=True):
        """Bracket the context's compute kernels with CUDA events."""
        self._check(self._lib.ztm_ctx_profile(self._h, 1 if enable else 0))

    def profile_read(self, name=""):
        """(total device ms, launches) of traced kernels matching `name`;
        clears the records."""
        ms = ctypes.c_double(0.0)
        n = ctypes.c_longlong(0)
        self._check(self._lib.ztm_ctx_profile_read(self._h, name.encode(), ctypes.byref(ms),
                                                   ctypes.byref(n)))
        return ms.value, n.value

    def tuning(self, max_rows=256):
        """The autotuner's timed candidates: rows of (stage KB, log2 pairs per
        item, kernel variant, microseconds) for batched launches."""
        buf = (ctypes.c_int * (4 * max_rows))()
        n = self._lib.ztm_ctx_tuning(self._h, buf, max_rows)
        if n < 0:
            raise GravityError(n, "bad argument")
        return [tuple(buf[4 * i:4 * i + 4]) for i in range(n)]

    def count_forms(self, enable=True):
        """Run the mixed forward's counting far kernel while enabled."""
        self._check(self._lib.ztm_ctx_count_forms(self._h, 1 if enable else 0))

    def form_counts(self):
        """(sixth-order slots, second-order slots, column-pair slots, near
        Phi evaluations) since the last read; clears them."""
        out = (ctypes.c_longlong * 4)()
        self._check(self._lib.ztm_ctx_form_counts(self._h, out))
        return tuple(int(v) for v in out)

    def test_timeout(self, polls):
        """Test hook of the timeout path: polls > 0 makes the far kernel's
        stage waits run out (on a barrier nothing completes); 0: off."""
        self._check(self._lib.ztm_ctx_test_timeout(self._h, int(polls)))

    def measure_peak(self, kind):
        """kind 'fp32' / 'fp64' (TFLOP/s of FMA) or 'rsqrt' (Gop/s)."""
        k = {"fp32": 0, "fp64": 1, "rsqrt": 2}[kind]
        v = ctypes.c_double(0.0)
        self._check(self._lib.ztm_measure_peak(self._h, k, ctypes.byref(v)))
        return v.value

    # -- point mass (TFM.cpp:90-99) -------------------------------------
    def pointmass(self, grid, drho, surf, nn=None, precision="fp64"):
        """G (di*dj, mGal) from drho (ii*jj*kk, g/cc) and surf (di*dj)."""
        ii = (grid.di - 1) * grid.fh + 1
        jj = (grid.dj - 1) * grid.fh + 1
        kk = (grid.dk - 1) * grid.fv + 1
        a = _Args(self)
        pd = a.arr(drho, ii * jj * kk, name="drho")
        ps = a.arr(surf, grid.di * grid.dj, name="surf")
        pn, n_nn = None, 0
        if nn is not None:
            pn = a.arr(nn, None, dtype=np.int32, name="nn")
            n_nn = int(nn.numel() if _is_torch_cuda(nn) else np.asarray(nn).size)
        out, po = a.out(grid.di * grid.dj, drho)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._run(a, self._lib.ztm_gfm_pointmass, self._h, ctypes.byref(grid), pd, pn, n_nn, ps, po,
                                                prec, a.flags)
        return out

    # -- density builder (TFM.cpp:83-89) -------------------------------
    def density(self, di, dj, dk, sea, M, v, vm, ro, dr, rc, fh=1, fv=2):
        """drho on the fine grid from the sea-level map, rendered Moho and
        velocity grids; returns (drho, number of selected nodes or -1)."""
        p = _lib.DensityParams(di, dj, dk, fh, fv, vm, ro, dr, (ctypes.c_double * 10)(*rc))
        N = ((di - 1) * fh + 1) * ((dj - 1) * fh + 1) * ((dk - 1) * fv + 1)
        a = _Args(self)
        ps = a.arr(sea, di * dj, name="sea")
        pm = a.arr(M, di * dj, name="M")
        pv = a.arr(v, di * dj * dk, name="v")
        out, po = a.out(N, sea)
        n = ctypes.c_longlong(0)
        self._run(a, self._lib.ztm_density_build, self._h, ctypes.byref(p), ps, pm, pv, po,
                                                ctypes.byref(n), a.flags)
        return out, n.value

    def pointmass_model(self, grid, sea, M, v, surf, vm, ro, dr, rc, precision="fp64"):
        """TFM.cpp:83-99 in one call: G (di*dj, mGal) from the sea-level map,
        rendered Moho and velocity grids, drho staying on the device."""
        p = _lib.DensityParams(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, vm, ro, dr,
                               (ctypes.c_double * 10)(*rc))
        a = _Args(self)
        ps = a.arr(sea, grid.di * grid.dj, name="sea")
        pm = a.arr(M, grid.di * grid.dj, name="M")
        pv = a.arr(v, grid.di * grid.dj * grid.dk, name="v")
        pf = a.arr(surf, grid.di * grid.dj, name="surf")
        out, po = a.out(grid.di * grid.dj, sea)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._run(a, self._lib.ztm_gfm_pointmass_model, self._h, ctypes.byref(p),
                  ctypes.byref(grid), ps, pm, pv, pf, po, prec, a.flags)
        return out

    # -- derivatives of the reference model (TFM.cpp:101-103, 124-135) -----
    def pointmass_adjoint(self, grid, surf, w, nn=None, drho=None, precision="fp64"):
        """J^T w: g[n] = sum over interior stations of w[m] dG[m]/d drho[n]
        for the nodes of nn (with multiplicity), else of |drho| > threshold
        when drho is given, else every node."""
        ii = (grid.di - 1) * grid.fh + 1
        jj = (grid.dj - 1) * grid.fh + 1
        kk = (grid.dk - 1) * grid.fv + 1
        a = _Args(self)
        ps = a.arr(surf, grid.di * grid.dj, name="surf")
        pw = a.arr(w, grid.di * grid.dj, name="w")
        pd = a.arr(drho, ii * jj * kk, name="drho") if drho is not None else None
        pn, n_nn = None, 0
        if nn is not None:
            pn = a.arr(nn, None, dtype=np.int32, name="nn")
            n_nn = int(nn.numel() if _is_torch_cuda(nn) else np.asarray(nn).size)
        out, po = a.out(ii * jj * kk, surf)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._run(a, self._lib.ztm_gfm_pointmass_adjoint, self._h, ctypes.byref(grid), pd, pn,
                  n_nn, ps, pw, po, prec, a.flags)
        return out

    def pointmass_misfit(self, grid, drho, surf, GD, g0=0.0, gsig=1.0, nn=None,
                         precision="fp64", gradient=True):
        """The gravity misfit of TFM.cpp:101-103.  Returns (ssq, res, G,
        g_drho, g_g0): res in TFM's order (i0 outer, j0 inner over the bfr
        interior), g_drho = d ssq / d drho and g_g0 = d ssq / d g0 (None
        without gradient)."""
        ii = (grid.di - 1) * grid.fh + 1
        jj = (grid.dj - 1) * grid.fh + 1
        kk = (grid.dk - 1) * grid.fv + 1
        ns = max(0, grid.di - 2 * grid.bfr) * max(0, grid.dj - 2 * grid.bfr)
        a = _Args(self)
        pd = a.arr(drho, ii * jj * kk, name="drho")
        ps = a.arr(surf, grid.di * grid.dj, name="surf")
        pgd = a.arr(GD, grid.di * grid.dj, name="GD")
        pn, n_nn = None, 0
        if nn is not None:
            pn = a.arr(nn, None, dtype=np.int32, name="nn")
            n_nn = int(nn.numel() if _is_torch_cuda(nn) else np.asarray(nn).size)
        res, pres = a.out(max(ns, 1), drho)
        G, pG = a.out(grid.di * grid.dj, drho)
        g, pg = a.out(ii * jj * kk, drho) if gradient else (None, None)
        ssq, pssq = a.scalar(drho)
        g0h, pg0 = a.scalar(drho) if gradient else (None, None)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._run(a, self._lib.ztm_gfm_pointmass_misfit, self._h, ctypes.byref(grid), pd, pn, n_nn,
                  ps, pgd, float(g0), float(gsig), pssq, pres, pG, pg, pg0, prec, a.flags)
        return (a.value(ssq), res[:ns], G, g, a.value(g0h) if gradient else None)

    def pointmass_model_misfit(self, grid, sea, M, v, surf, GD, vm, ro, dr, rc, g0=0.0, gsig=1.0,
                               precision="fp64", gradient=True):
        """TFM.cpp:83-103 with the gradient chained through the density
        builder.  Returns a dict: ssq, res, G and, with gradient, g_M
        (d ssq / d M), g_v (d ssq / d v) and g_par (d ssq / d (vm, ro, dr, g0))."""
        p = _lib.DensityParams(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, vm, ro, dr,
                               (ctypes.c_double * 10)(*rc))
        ns = max(0, grid.di - 2 * grid.bfr) * max(0, grid.dj - 2 * grid.bfr)
        M2 = grid.di * grid.dj
        a = _Args(self)
        pse = a.arr(sea, M2, name="sea")
        pm = a.arr(M, M2, name="M")
        pv = a.arr(v, M2 * grid.dk, name="v")
        pf = a.arr(surf, M2, name="surf")
        pgd = a.arr(GD, M2, name="GD")
        res, pres = a.out(max(ns, 1), sea)
        G, pG = a.out(M2, sea)
        if gradient:
            gM, pgM = a.out(M2, sea)
            gv, pgv = a.out(M2 * grid.dk, sea)
            gp, pgp = a.out(4, sea)
        else:
            gM = gv = gp = None
            pgM = pgv = pgp = None
        ssq, pssq = a.scalar(sea)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._run(a, self._lib.ztm_gfm_pointmass_model_misfit, self._h, ctypes.byref(p),
                  ctypes.byref(grid), pse, pm, pv, pf, pgd, float(g0), float(gsig), pssq, pres, pG,
                  pgM, pgv, pgp, prec, a.flags)
        out = {"ssq": a.value(ssq), "res": res[:ns], "G": G}
        if gradient:
            out.update(g_M=gM, g_v=gv, g_par=gp)
        return out

    # -- prism mesh -----------------------------------------------------
    def prism(self, mesh, rho, stations, precision="mixed", G=None, near_q=None, tile=0, chunk=0,
              autotune=False):
        np_ = mesh.nx * mesh.ny * mesh.nz
        a = _Args(self)
        pr = a.arr(rho, np_, name="rho")
        ns = _nstations(stations)
        px = a.arr(stations, 3 * ns, name="stations")
        out, po = a.out(ns, rho)
        o = _opts(precision, a.flags | (AUTOTUNE if autotune else 0), G, near_q, tile, chunk)
        self._run(a, self._lib.ztm_gfm_prism, self._h, ctypes.byref(mesh), pr, ns, px, po,
                                            ctypes.byref(o))
        return out

    def prism_list(self, geom, rho, stations, precision="fp64", G=None, near_q=None):
        n = _nstations_list(geom)
        a = _Args(self)
        pg = a.arr(geom, 6 * n, name="geom")
        pr = a.arr(rho, n, name="rho")
        ns = _nstations(stations)
        px = a.arr(stations, 3 * ns, name="stations")
        out, po = a.out(ns, rho)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_prism_list, self._h, n, pg, pr, ns, px, po, ctypes.byref(o))
        return out

    def adjoint(self, mesh, stations, resid, precision="mixed", G=None, near_q=None):
        np_ = mesh.nx * mesh.ny * mesh.nz
        ns = _nstations(stations)
        a = _Args(self)
        px = a.arr(stations, 3 * ns, name="stations")
        pr = a.arr(resid, ns, name="resid")
        out, po = a.out(np_, resid)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_adjoint, self._h, ctypes.byref(mesh), ns, px, pr, po,
                                              ctypes.byref(o))
        return out

    # -- interface --------------------------------------------------------
    def interface(self, imesh, depth, rho_col, stations, precision="mixed", G=None, near_q=None):
        nc = imesh.nx * imesh.ny
        ns = _nstations(stations)
        a = _Args(self)
        pd = a.arr(depth, nc, name="depth")
        pr = a.arr(rho_col, nc, name="rho_col")
        px = a.arr(stations, 3 * ns, name="stations")
        out, po = a.out(ns, depth)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_interface, self._h, ctypes.byref(imesh), pd, pr, ns, px, po,
                                                ctypes.byref(o))
        return out

    def interface_adjoint(self, imesh, depth, rho_col, stations, resid, precision="mixed",
                          G=None, near_q=None):
        nc = imesh.nx * imesh.ny
        ns = _nstations(stations)
        a = _Args(self)
        pd = a.arr(depth, nc, name="depth")
        pr = a.arr(rho_col, nc, name="rho_col")
        px = a.arr(stations, 3 * ns, name="stations")
        pres = a.arr(resid, ns, name="resid")
        g_rho, pgr = a.out(nc, depth)
        g_dep, pgd = a.out(nc, depth)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_interface_adjoint, self._h, ctypes.byref(imesh), pd, pr, ns,
                                                        px, pres, pgr, pgd, ctypes.byref(o))
        return g_rho, g_dep

    def interface_jvp(self, imesh, depth, rho_col, stations, d_depth, precision="mixed", G=None,
                      near_q=None):
        """dgz = J_depth d_depth: the change of gz (mGal) per unit step along
        d_depth (metres), without forming J."""
        nc = imesh.nx * imesh.ny
        ns = _nstations(stations)
        a = _Args(self)
        pd = a.arr(depth, nc, name="depth")
        pr = a.arr(rho_col, nc, name="rho_col")
        pv = a.arr(d_depth, nc, name="d_depth")
        px = a.arr(stations, 3 * ns, name="stations")
        out, po = a.out(ns, depth)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_interface_jvp, self._h, ctypes.byref(imesh), pd, pr, pv, ns,
                  px, po, ctypes.byref(o))
        return out

    def interface_misfit(self, imesh, depth, rho_col, stations, data, precision="mixed",
                         G=None, near_q=None):
        """Returns (misfit, gz, g_rho, g_depth) for misfit 0.5*|gz - data|^2."""
        nc = imesh.nx * imesh.ny
        ns = _nstations(stations)
        a = _Args(self)
        pd = a.arr(depth, nc, name="depth")
        pr = a.arr(rho_col, nc, name="rho_col")
        px = a.arr(stations, 3 * ns, name="stations")
        pdat = a.arr(data, ns, name="data")
        gz, pgz = a.out(ns, depth)
        g_rho, pgr = a.out(nc, depth)
        g_dep, pgd = a.out(nc, depth)
        mis = ctypes.c_double(0.0)
        if a.device:
            import torch
            mt = torch.zeros(1, dtype=torch.float64, device=depth.device)
            a.keep.append(mt)
            pmis = ctypes.c_void_p(mt.data_ptr())
        else:
            pmis = ctypes.cast(ctypes.pointer(mis), ctypes.c_void_p)
        o = _opts(precision, a.flags, G, near_q)
        self._run(a, self._lib.ztm_gfm_interface_misfit, self._h, ctypes.byref(imesh), pd, pr, ns,
                                                       px, pdat, pmis, pgz, pgr, pgd,
                                                       ctypes.byref(o))
        misfit = mt if a.device else mis.value
        return misfit, gz, g_rho, g_dep

    def invert_interface(self, imesh, depth0, rho_col, stations, data, lam=1e-2, iterations=20,
                         precision="mixed", G=None, near_q=None, method="lbfgs", cg_iterations=10):
        """Inversion of the column tops (host arrays) by L-BFGS (method
        "lbfgs") or Gauss-Newton with CG inner solves ("gn").  Returns
        (depth, data-misfit history, iterations taken)."""
        nc = imesh.nx * imesh.ny
        ns = _nstations(stations)
        a = _Args(self)
        depth = np.array(depth0, dtype=np.float64, copy=True)
        if depth.size != nc:
            raise ValueError("depth0 has %d values, expected %d" % (depth.size, nc))
        pd = depth.ctypes.data_as(ctypes.c_void_p)
        pr = a.arr(rho_col, nc, name="rho_col")
        px = a.arr(stations, 3 * ns, name="stations")
        pdat = a.arr(data, ns, name="data")
        if a.device:
            raise ValueError("invert_interface takes host arrays")
        hist = np.zeros(iterations + 1)
        done = ctypes.c_int(0)
        o = _opts(precision, 0, G, near_q)
        ph = hist.ctypes.data_as(ctypes.c_void_p)
        if method == "gn":
            self._check(self._lib.ztm_invert_interface_gn(self._h, ctypes.byref(imesh), pd, pr, ns,
                                                          px, pdat, float(lam), int(iterations),
                                                          int(cg_iterations), ctypes.byref(o), ph,
                                                          ctypes.byref(done)))
        elif method == "lbfgs":
            self._check(self._lib.ztm_invert_interface(self._h, ctypes.byref(imesh), pd, pr, ns, px,
                                                       pdat, float(lam), int(iterations),
                                                       ctypes.byref(o), ph, ctypes.byref(done)))
        else:
            raise ValueError("method must be 'lbfgs' or 'gn'")
        return depth, hist[:done.value + 1], done.value

    # -- damped Gauss-Newton step (TFM.cpp:159-160) -------------------------
    def lm_steps(self, J, r, b, sig, damping, return_jtj=False):
        """The trial models b + inv(J^T J + d0 diag(J^T J) + d1 diag(1/sig^2))
        J^T r for each damping pair (d0, d1); J is (nrows, ncols).  Returns
        B (nd, ncols) and, with return_jtj, J^T J."""
        shape = tuple(J.shape)
        if len(shape) != 2:
            raise ValueError("J must be (nrows, ncols)")
        nrows, ncols = int(shape[0]), int(shape[1])
        nd = int(damping.shape[0]) if len(tuple(damping.shape)) == 2 else int(damping.shape[0]) // 2
        a = _Args(self)
        pJ = a.arr(J, nrows * ncols, name="J")
        pr = a.arr(r, nrows, name="r")
        pb = a.arr(b, ncols, name="b")
        ps = a.arr(sig, ncols, name="sig")
        pd = a.arr(damping, 2 * nd, name="damping")
        B, pB = a.out(nd * ncols, J)
        JJ, pJJ = a.out(ncols * ncols, J) if return_jtj else (None, None)
        self._run(a, self._lib.ztm_lm_steps, self._h, pJ, nrows, ncols, pr, pb, ps, pd, nd, pB, pJJ,
                  a.flags)
        B = B.reshape(nd, ncols)
        return (B, JJ.reshape(ncols, ncols)) if return_jtj else B

    # -- batched ----------------------------------------------------------
    def batch(self, jobs, precision="mixed", G=None, near_q=None, autotune=False):
        """jobs: list of (mesh, rho[nmodels, nprisms], stations[ns, 3]).
        Returns a list of gz arrays [nmodels, ns].  autotune: the first call
        for these job shapes times the candidate launch shapes and keeps the
        fastest on the context."""
        a = _Args(self)
        arr = (_lib.Job * len(jobs))()
        outs = []
        for i, (mesh, rho, st) in enumerate(jobs):
            np_ = mesh.nx * mesh.ny * mesh.nz
            nm = int(rho.shape[0]) if getattr(rho, "ndim", 1) == 2 else 1
            ns = _nstations(st)
            pr = a.arr(rho, nm * np_, name="rho")
            px = a.arr(st, 3 * ns, name="stations")
            out, po = a.out(nm * ns, rho)
            outs.append((out, nm, ns))
            arr[i].mesh = mesh
            arr[i].nmodels = nm
            arr[i].rho = pr
            arr[i].ns = ns
            arr[i].sxyz = px
            arr[i].gz = po
        o = _opts(precision, a.flags | (AUTOTUNE if autotune else 0), G, near_q)
        self._run(a, self._lib.ztm_gfm_batch, self._h, arr, len(jobs), ctypes.byref(o))
        return [out.reshape(nm, ns) for out, nm, ns in outs]


def _nstations(st):
    shape = tuple(st.shape)
    if len(shape) == 2 and shape[1] == 3:
        return int(shape[0])
    if len(shape) == 1 and shape[0] % 3 == 0:
        return int(shape[0] // 3)
    raise ValueError("stations must be (ns, 3)")


def _nstations_list(geom):
    shape = tuple(geom.shape)
    if len(shape) == 2 and shape[1] == 6:
        return int(shape[0])
    if len(shape) == 1 and shape[0] % 6 == 0:
        return int(shape[0] // 6)
    raise ValueError("geom must be (np, 6)")
