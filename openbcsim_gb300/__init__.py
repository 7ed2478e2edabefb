"""GB300-native COLE ultrasound line simulator.

`RfSimulator` mirrors the reference's Python class `pyrfsim.RfSimulator`
(src/python/PythonInterface.cpp:58-351): the same method names, argument
meanings, array shapes and error messages, over the C ABI of
include/bcsim_gb300.h.  Errors raise RuntimeError with the reference's message.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _capi

__all__ = ["RfSimulator", "Batch", "Server", "SimulatorError", "load_library", "configure_job"]


class SimulatorError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def load_library():
    return _capi.load()


def _f32(a, shape_msg: str, ndim: int, last: Optional[int] = None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if arr.ndim != ndim:
        raise RuntimeError(shape_msg)
    if last is not None and arr.shape[-1] != last:
        raise RuntimeError(shape_msg)
    return arr


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class RfSimulator:
    """One simulator instance (`bcsim::Create(sim_type)`, LibBCSim.cpp:39-49)."""

    def __init__(self, sim_type: str = "gpu"):
        self._lib = _capi.load()
        h = C.c_void_p()
        rc = self._lib.bcsim_create(sim_type.encode(), C.byref(h))
        if rc != 0:
            raise SimulatorError(rc, self._lib.bcsim_last_error(None).decode())
        self._h = h
        self._print_debug = False
        self._log_cb = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.bcsim_destroy(h)
            self._h = None

    def _check(self, rc: int):
        if rc != 0:
            raise SimulatorError(rc, self._lib.bcsim_last_error(self._h).decode())

    @property
    def handle(self):
        return self._h

    # --- PythonInterface.cpp:70-78 ---
    def set_print_debug(self, val: bool):
        self._print_debug = bool(val)

    def set_parameter(self, key: str, value: str):
        self._check(self._lib.bcsim_set_parameter(self._h, key.encode(), str(value).encode()))

    def get_parameter(self, key: str) -> str:
        buf = C.create_string_buffer(1024)
        self._check(self._lib.bcsim_get_parameter(self._h, key.encode(), buf, 1024))
        return buf.value.decode()

    # --- fixed scatterers, PythonInterface.cpp:80-101: data [N, 4] ---
    def clear_fixed_scatterers(self):
        self._check(self._lib.bcsim_clear_fixed_scatterers(self._h))

    def add_fixed_scatterers(self, data):
        arr = np.asarray(data)
        if arr.ndim != 2 or arr.shape[1] != 4:
            raise RuntimeError("add_fixed_scatterers : Number of columns must be four")
        arr = np.ascontiguousarray(arr, dtype=np.float32)
        self._check(self._lib.bcsim_add_fixed_scatterers(self._h, _ptr(arr), arr.shape[0]))

    # --- spline scatterers, PythonInterface.cpp:103-177 ---
    def clear_spline_scatterers(self):
        self._check(self._lib.bcsim_clear_spline_scatterers(self._h))

    def add_spline_scatterers(self, spline_degree: int, knot_vector, control_points, amplitudes):
        knots = np.asarray(knot_vector)
        if knots.ndim != 1:
            raise RuntimeError("add_spline_scatterers : invalid knot vector rank")
        cps = np.asarray(control_points)
        if cps.ndim != 3:
            raise RuntimeError("add_spline_scatterers : invalid control_points rank")
        n, k = cps.shape[0], cps.shape[1]
        if len(knots) != k + int(spline_degree) + 1:
            raise RuntimeError("add_spline_scatterers : mismatch in number of nodes, degree and control points")
        if cps.shape[2] != 3:
            raise RuntimeError("add_spline_scatterers : size of dimension 3 must be three (x,y,z)")
        amps = np.asarray(amplitudes)
        if amps.shape[0] != n:
            raise RuntimeError("Mismatch between control_points and amplitudes")
        knots = np.ascontiguousarray(knots, np.float32)
        cps = np.ascontiguousarray(cps, np.float32)
        amps = np.ascontiguousarray(amps, np.float32)
        self._check(self._lib.bcsim_add_spline_scatterers(self._h, int(spline_degree), _ptr(knots), len(knots),
                                                          _ptr(cps), _ptr(amps), n, k))

    # --- scan sequence, PythonInterface.cpp:179-220 ---
    def set_scan_sequence(self, origins, directions, line_length, lateral_dirs, timestamps):
        o = np.asarray(origins)
        d = np.asarray(directions)
        l = np.asarray(lateral_dirs)
        t = np.asarray(timestamps)
        if o.ndim != 2 or d.ndim != 2 or l.ndim != 2 or t.ndim != 1:
            raise RuntimeError("set_scan_sequence(): Invalid rank.")
        n = o.shape[0]
        if n != d.shape[0] or n != l.shape[0]:
            raise RuntimeError("set_scan_sequence(): Mismatch in number of rows.")
        o, d, l, t = (np.ascontiguousarray(x, np.float32) for x in (o, d, l, t))
        self._check(self._lib.bcsim_set_scan_sequence(self._h, _ptr(o), _ptr(d), _ptr(l), _ptr(t), n,
                                                      float(line_length)))

    # --- excitation, PythonInterface.cpp:222-241 ---
    def set_excitation(self, samples, center_index: int, fs: float, demod_freq: float):
        s = np.asarray(samples)
        if s.ndim != 1:
            raise RuntimeError("set_excitation: samples should be one-dimensional")
        s = np.ascontiguousarray(s, np.float32)
        self._check(self._lib.bcsim_set_excitation(self._h, _ptr(s), len(s), int(center_index), float(fs),
                                                   float(demod_freq)))

    # --- beam profiles, PythonInterface.cpp:243-297 ---
    def set_analytical_beam_profile(self, sigma_lateral: float, sigma_elevational: float):
        self._check(self._lib.bcsim_set_analytical_profile(self._h, float(sigma_lateral), float(sigma_elevational)))

    def set_lut_beam_profile(self, r_min, r_max, l_min, l_max, e_min, e_max, samples):
        s = np.asarray(samples)
        if s.ndim != 3:
            raise RuntimeError("Number of sample dimensions must be three.")
        s = np.ascontiguousarray(s, np.float32)
        self._check(self._lib.bcsim_set_lookup_profile(self._h, _ptr(s), s.shape[0], s.shape[1], s.shape[2],
                                                       r_min, r_max, l_min, l_max, e_min, e_max))

    # --- simulate, PythonInterface.cpp:299-318: returns [num_samples, num_lines] complex64 ---
    def simulate_lines(self) -> np.ndarray:
        return self.simulate_lines_line_major().T

    def simulate_lines_line_major(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """IQ as [num_lines, num_samples] complex64 (the C ABI's layout)."""
        L, nd = C.c_int64(), C.c_int64()
        self._check(self._lib.bcsim_get_output_shape(self._h, C.byref(L), C.byref(nd)))
        if out is None or out.shape != (L.value, nd.value) or out.dtype != np.complex64:
            out = np.empty((L.value, nd.value), np.complex64)
        self._check(self._lib.bcsim_simulate_lines(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size,
                                                   C.byref(L), C.byref(nd)))
        return out

    def simulate_fixed_frames(self, frames, outs=None):
        """A stream of fixed-scatterer frames (each [n, 4] float32, the same n),
        each replacing the fixed datasets: returns (or fills) one IQ array
        [num_lines, num_samples] complex64 per frame, bit for bit what
        clear_fixed_scatterers + add_fixed_scatterers + simulate_lines_line_major
        per frame give.  The next frame's upload overlaps the current frame's
        simulation (pinned host arrays let the copies run asynchronously)."""
        frames = [_f32(f, "frames must be [n, 4] float32 arrays", 2, 4) for f in frames]
        if not frames:
            return []
        n = frames[0].shape[0]
        if any(f.shape[0] != n for f in frames):
            raise ValueError("every frame must hold the same number of scatterers")
        L, nd = self.output_shape()
        if outs is None:
            outs = [np.empty((L, nd), np.complex64) for _ in frames]
        if len(outs) != len(frames) or any(o.shape != (L, nd) or o.dtype != np.complex64 or
                                           not o.flags.c_contiguous for o in outs):
            raise ValueError("outs must hold one C-contiguous complex64 [num_lines, num_samples] array per frame")
        fp = (C.POINTER(C.c_float) * len(frames))(*[f.ctypes.data_as(C.POINTER(C.c_float)) for f in frames])
        op = (C.POINTER(C.c_float) * len(outs))(*[o.ctypes.data_as(C.POINTER(C.c_float)) for o in outs])
        self._check(self._lib.bcsim_simulate_fixed_frames(self._h, fp, n, len(frames), op, L * nd))
        return outs

    def simulate_spline_frames(self, degree, knots, cps_frames, amps_frames, outs=None):
        """A stream of spline frames of one shape: frame k's control points
        cps_frames[k] ([n, num_cs, 3] float32) and amplitudes amps_frames[k] ([n]
        float32), with the given degree and knots, replace the spline datasets;
        returns (or fills) one IQ array [num_lines, num_samples] complex64 per
        frame, bit for bit what clear_spline_scatterers + add_spline_scatterers +
        simulate_lines_line_major per frame give.  The next frame's upload
        overlaps the current frame's simulation (pinned host arrays let the
        copies run asynchronously)."""
        knots = np.ascontiguousarray(knots, np.float32)
        cps_frames = [np.ascontiguousarray(c) for c in cps_frames]
        amps_frames = [np.ascontiguousarray(a) for a in amps_frames]
        if not cps_frames:
            return []
        if len(amps_frames) != len(cps_frames):
            raise ValueError("one amplitude array per frame")
        shape = cps_frames[0].shape
        if len(shape) != 3 or shape[2] != 3:
            raise ValueError("control points must be [n, num_cs, 3] float32 arrays")
        n, num_cs = shape[0], shape[1]
        for c, a in zip(cps_frames, amps_frames):
            if c.dtype != np.float32 or c.shape != shape or a.dtype != np.float32 or a.shape != (n,):
                raise ValueError("every frame must hold float32 [n, num_cs, 3] control points and [n] amplitudes")
        L, nd = self.output_shape()
        if outs is None:
            outs = [np.empty((L, nd), np.complex64) for _ in cps_frames]
        if len(outs) != len(cps_frames) or any(o.shape != (L, nd) or o.dtype != np.complex64 or
                                               not o.flags.c_contiguous for o in outs):
            raise ValueError("outs must hold one C-contiguous complex64 [num_lines, num_samples] array per frame")
        f = C.POINTER(C.c_float)
        cp = (f * len(cps_frames))(*[c.ctypes.data_as(f) for c in cps_frames])
        ap = (f * len(amps_frames))(*[a.ctypes.data_as(f) for a in amps_frames])
        op = (f * len(outs))(*[o.ctypes.data_as(f) for o in outs])
        self._check(self._lib.bcsim_simulate_spline_frames(self._h, int(degree), knots.ctypes.data_as(f),
                                                           knots.size, cp, ap, n, num_cs, len(cps_frames), op,
                                                           L * nd))
        return outs

    def simulate_lines_device(self, device_ptr: int, capacity: int):
        """IQ into a device buffer of `capacity` complex64 values (no host copy)."""
        self._check(self._lib.bcsim_simulate_lines_device(self._h, C.c_void_p(device_ptr), int(capacity)))

    def output_shape(self):
        L, nd = C.c_int64(), C.c_int64()
        self._check(self._lib.bcsim_get_output_shape(self._h, C.byref(L), C.byref(nd)))
        return L.value, nd.value

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.bcsim_get_stream(self._h, C.byref(s)))
        return s.value or 0

    # --- PythonInterface.cpp:320-337 ---
    def get_debug_data(self, identifier: str):
        n = C.c_int64()
        buf = (C.c_double * 65536)()
        self._check(self._lib.bcsim_get_debug_data(self._h, identifier.encode(), buf, 65536, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def get_total_num_scatterers(self) -> int:
        n = C.c_int64()
        self._check(self._lib.bcsim_get_total_num_scatterers(self._h, C.byref(n)))
        return n.value

    # --- post-processing on the device (RefreshWorker.hpp:179-395) ---
    def bmode_image(self, iq, dyn_range: float = 60.0, gain: float = 1.0, normalize: float = 0.0,
                    geometry: Optional["ScanGeometry"] = None, beamspace: bool = False):
        """B-mode of an IQ frame iq [num_lines, num_samples] complex64: log-compressed
        beam-space bytes and, with a geometry, the scan-converted image [ny, nx]
        uint8.  normalize <= 0 normalises by the frame's largest envelope.
        Returns (image or None, beamspace or None, normalize_used)."""
        iq = np.ascontiguousarray(iq, np.complex64)
        if iq.ndim != 2:
            raise ValueError("iq must be [num_lines, num_samples]")
        return self._bmode(iq, dyn_range, gain, normalize, geometry, beamspace)

    def simulate_bmode(self, dyn_range: float = 60.0, gain: float = 1.0, normalize: float = 0.0,
                       geometry: Optional["ScanGeometry"] = None, beamspace: bool = False):
        """simulate_lines followed by bmode_image, the IQ staying on the device."""
        return self._bmode(None, dyn_range, gain, normalize, geometry, beamspace)

    def _bmode(self, iq, dyn_range, gain, normalize, geometry, beamspace):
        L, nd = (iq.shape if iq is not None else self.output_shape())
        g = geometry.c_struct() if geometry is not None else None
        image = np.empty((geometry.ny, geometry.nx), np.uint8) if geometry is not None else None
        bs = np.empty((L, nd), np.uint8) if beamspace else None
        used = C.c_float()
        gp = C.byref(g) if g is not None else None
        ip = image.ctypes.data_as(C.c_void_p) if image is not None else None
        bp = bs.ctypes.data_as(C.c_void_p) if bs is not None else None
        if iq is not None:
            self._check(self._lib.bcsim_bmode_image(self._h, iq.ctypes.data_as(C.POINTER(C.c_float)), L, nd,
                                                    dyn_range, gain, normalize, gp, ip, bp, C.byref(used)))
        else:
            self._check(self._lib.bcsim_simulate_bmode(self._h, dyn_range, gain, normalize, gp, ip, bp,
                                                       C.byref(used)))
        return image, bs, used.value

    def scan_convert(self, beamspace, geometry: "ScanGeometry") -> np.ndarray:
        """Scan conversion of a float beam space [num_beams, num_range] into [ny, nx] float32."""
        b = np.ascontiguousarray(beamspace, np.float32)
        out = np.empty((geometry.ny, geometry.nx), np.float32)
        g = geometry.c_struct()
        self._check(self._lib.bcsim_scan_convert(self._h, _ptr(b), b.shape[0], b.shape[1], C.byref(g), _ptr(out)))
        return out

    def simulate_packet(self, packet_size: int, prt: float) -> np.ndarray:
        """A colour-Doppler packet: [packet_size, num_lines, num_samples] complex64, frame k
        with every timestamp advanced by k * prt."""
        L, nd = self.output_shape()
        out = np.empty((packet_size, L, nd), np.complex64)
        self._check(self._lib.bcsim_simulate_packet(self._h, packet_size, prt,
                                                    out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def color_doppler(self, iq_packet, geometry: Optional["ScanGeometry"] = None):
        """R0 and velocity (arg R1) [num_lines, num_samples] float32 of a packet
        [P, num_lines, num_samples], and with a geometry the colour image [ny, nx, 4]
        (blue, green, red, alpha).  Returns (r0, velocity, image or None)."""
        p = np.ascontiguousarray(iq_packet, np.complex64)
        if p.ndim != 3:
            raise ValueError("iq_packet must be [packet_size, num_lines, num_samples]")
        return self._doppler(p, 0, 0.0, geometry)

    def simulate_color_doppler(self, packet_size: int, prt: float, geometry: Optional["ScanGeometry"] = None):
        """simulate_packet followed by color_doppler, on the device."""
        return self._doppler(None, packet_size, prt, geometry)

    def _doppler(self, packet, packet_size, prt, geometry):
        L, nd = (packet.shape[1:] if packet is not None else self.output_shape())
        r0 = np.empty((L, nd), np.float32)
        vel = np.empty((L, nd), np.float32)
        g = geometry.c_struct() if geometry is not None else None
        img = np.empty((geometry.ny, geometry.nx, 4), np.uint8) if geometry is not None else None
        gp = C.byref(g) if g is not None else None
        ip = img.ctypes.data_as(C.c_void_p) if img is not None else None
        if packet is not None:
            self._check(self._lib.bcsim_color_doppler(self._h, packet.ctypes.data_as(C.POINTER(C.c_float)),
                                                      packet.shape[0], L, nd, _ptr(r0), _ptr(vel), gp, ip))
        else:
            self._check(self._lib.bcsim_simulate_color_doppler(self._h, packet_size, prt, _ptr(r0), _ptr(vel), gp,
                                                               ip))
        return r0, vel, img

    def debug_raise_wait_flag(self):
        """Test hook: set the device error flag as a bounded wait that gave up
        would; the next synchronising call fails and clears it."""
        self._check(self._lib.bcsim_debug_raise_wait_flag(self._h))

    def set_logger(self, fn):
        """fn(level: int, message: str) receives the engine's log messages; None silences."""
        if fn is None:
            self._log_cb = None
            self._check(self._lib.bcsim_set_logger(self._h, _capi.LOG_FN(), None))
            return
        self._log_cb = _capi.LOG_FN(lambda lvl, msg, user: fn(int(lvl), msg.decode()))
        self._check(self._lib.bcsim_set_logger(self._h, self._log_cb, None))


class ScanGeometry:
    """A sector or linear scan geometry with the output image size
    (bcsim::SectorScanGeometry / LinearScanGeometry, src/utils/ScanGeometry.hpp:44-78)."""

    def __init__(self, kind: str, width: float, depth: float, nx: int, ny: int, tilt: float = 0.0):
        if kind not in ("sector", "linear"):
            raise ValueError("kind must be 'sector' or 'linear'")
        self.kind, self.width, self.depth, self.tilt, self.nx, self.ny = kind, width, depth, tilt, int(nx), int(ny)

    @staticmethod
    def image_size(kind: str, width: float, depth: float, dots_per_meter: float, tilt: float = 0.0):
        """(nx, ny) the reference's worker uses: the Cartesian extent in metres times
        dots per metre, truncated (RefreshWorker.hpp:192-199, ScanGeometry.hpp:49-55)."""
        from . import _imaging_host as H
        return H.image_size(kind, width, depth, dots_per_meter, tilt)

    def c_struct(self):
        return _capi.ScanGeometryC(_capi.GEOMETRY_SECTOR if self.kind == "sector" else _capi.GEOMETRY_LINEAR,
                                   self.width, self.depth, self.tilt, self.nx, self.ny)


def configure_job(sim: RfSimulator, job, precision_mode: str = "fp64"):
    """Configure a simulator from a workloads.Job (synthetic seeded inputs)."""
    sim.set_parameter("sound_speed", repr(float(np.float32(job.sound_speed))))
    sim.set_parameter("use_arc_projection", "on" if job.arc else "off")
    sim.set_parameter("phase_delay", "on" if job.phase_delay else "off")
    sim.set_parameter("radial_decimation", str(job.decimation))
    sim.set_parameter("precision_mode", precision_mode)
    if getattr(job, "noise_amplitude", 0.0):
        sim.set_parameter("noise_amplitude", repr(float(job.noise_amplitude)))
        # the seed resets the simulator's frame counter; its next simulation draws frame 0
        sim.set_parameter("noise_seed", str(int(job.noise_seed)))
    sim.set_excitation(job.taps, job.center_index, job.fs, job.demod_freq)
    s = job.scan
    sim.set_scan_sequence(s.origins, s.directions, s.line_length, s.lateral_dirs, s.timestamps)
    b = job.beam
    if hasattr(b, "sigma_lateral"):
        sim.set_analytical_beam_profile(b.sigma_lateral, b.sigma_elevational)
    else:
        sim.set_lut_beam_profile(b.r_range[0], b.r_range[1], b.l_range[0], b.l_range[1], b.e_range[0], b.e_range[1],
                                 b.samples)
    sim.clear_fixed_scatterers()
    for f in job.fixed:
        sim.add_fixed_scatterers(f.xyza)
    sim.clear_spline_scatterers()
    for sp in job.splines:
        sim.add_spline_scatterers(sp.degree, sp.knots, sp.control_points, sp.amplitudes)
    return sim


class Batch:
    """Several configured simulators run together (include/bcsim_gb300.h,
    bcsim_batch_*): all of their device work is submitted at once on separate
    streams and, from the second unchanged run on, replayed as one CUDA graph."""

    def __init__(self, sims, use_graph: bool = True):
        self._lib = _capi.load()
        self._sims = list(sims)
        arr = (C.c_void_p * len(self._sims))(*[s.handle.value for s in self._sims])
        b = C.c_void_p()
        rc = self._lib.bcsim_batch_create(arr, len(self._sims), int(use_graph), C.byref(b))
        if rc != 0:
            raise SimulatorError(rc, "bcsim_batch_create failed")
        self._b = b

    def __del__(self):
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            self._lib.bcsim_batch_destroy(b)
            self._b = None

    def run(self, outputs=None):
        """Run every job; returns (or fills) one [lines, samples] complex64 array per job."""
        if outputs is None:
            outputs = [np.empty(s.output_shape(), np.complex64) for s in self._sims]
        ptrs = (C.c_void_p * len(outputs))(*[o.ctypes.data for o in outputs])
        caps = (C.c_int64 * len(outputs))(*[o.size for o in outputs])
        rc = self._lib.bcsim_batch_run(self._b, ptrs, caps)
        if rc != 0:
            raise SimulatorError(rc, self._lib.bcsim_batch_last_error(self._b).decode())
        return outputs

    def run_device(self, device_ptrs, capacities) -> int:
        """Run into device buffers without waiting; returns the completion stream."""
        ptrs = (C.c_void_p * len(device_ptrs))(*device_ptrs)
        caps = (C.c_int64 * len(capacities))(*capacities)
        st = C.c_void_p()
        rc = self._lib.bcsim_batch_run_device(self._b, ptrs, caps, C.byref(st))
        if rc != 0:
            raise SimulatorError(rc, self._lib.bcsim_batch_last_error(self._b).decode())
        return st.value or 0


class Server:
    """Continuous-batching request server over resident phantoms
    (include/bcsim_gb300.h, bcsim_server_*)."""

    def __init__(self, hbm_budget_bytes: int = 16 << 30, max_slots_per_phantom: int = 4, max_in_flight: int = 3):
        self._lib = _capi.load()
        s = C.c_void_p()
        rc = self._lib.bcsim_server_create(int(hbm_budget_bytes), int(max_slots_per_phantom), C.byref(s))
        if rc != 0:
            raise SimulatorError(rc, "bcsim_server_create failed")
        self._s = s
        self._shapes = {}
        self._check(self._lib.bcsim_server_set_max_in_flight(self._s, int(max_in_flight)))

    def close(self):
        s = getattr(self, "_s", None)
        if s is not None and s.value:
            self._lib.bcsim_server_destroy(s)
            self._s = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise SimulatorError(rc, self._lib.bcsim_server_last_error(self._s).decode())

    def add_phantom(self, sim: RfSimulator) -> int:
        pid = C.c_int()
        self._check(self._lib.bcsim_server_add_phantom(self._s, sim.handle, C.byref(pid)))
        return pid.value

    def submit(self, phantom: int, origins, directions, line_length, lateral_dirs, timestamps, decimation: int) -> int:
        o, d, l, t = (np.ascontiguousarray(x, np.float32) for x in (origins, directions, lateral_dirs, timestamps))
        rid = C.c_int64()
        self._check(self._lib.bcsim_server_submit(self._s, int(phantom), _ptr(o), _ptr(d), _ptr(l), _ptr(t),
                                                  o.shape[0], float(line_length), int(decimation), C.byref(rid)))
        self._shapes[rid.value] = o.shape[0]
        return rid.value

    def wait(self, request_id: int, max_samples: int = 1 << 16, timeout_ms: int = -1):
        """(IQ [lines, samples] complex64, latency in ms) of a finished request."""
        L = self._shapes.get(request_id, 1)
        buf = np.empty(L * max_samples, np.complex64)
        nl, nd, lat = C.c_int64(), C.c_int64(), C.c_double()
        rc = self._lib.bcsim_server_wait(self._s, int(request_id), buf.ctypes.data_as(C.POINTER(C.c_float)),
                                         buf.size, C.byref(nl), C.byref(nd), C.byref(lat), int(timeout_ms))
        self._check(rc)
        self._shapes.pop(request_id, None)
        return buf[: nl.value * nd.value].reshape(nl.value, nd.value).copy(), lat.value

    INJECT_WAIT_FLAG, INJECT_WORKER_THROW, INJECT_FREE_MEMORY_CAP = 1, 2, 3

    def debug_inject(self, what: int, value: int = 0):
        """Test hook (bcsim_server_debug_inject): host-side fault injection."""
        self._check(self._lib.bcsim_server_debug_inject(self._s, int(what), int(value)))

    def stats(self) -> dict:
        c, f, q, pr, hb, qd = (C.c_int64() for _ in range(6))
        p50, p99 = C.c_double(), C.c_double()
        self._check(self._lib.bcsim_server_stats(self._s, C.byref(c), C.byref(f), C.byref(p50), C.byref(p99),
                                                 C.byref(pr), C.byref(hb), C.byref(qd)))
        return {"completed": c.value, "failed": f.value, "p50_ms": p50.value, "p99_ms": p99.value,
                "projections": pr.value, "hbm_in_use": hb.value, "queue_depth": qd.value}
