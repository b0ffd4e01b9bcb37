"""Batched ensemble engine over CDKLM16 members.

The reference steps its ensembles member by member from Python
(E/OceanNoiseEnsemble.py:517-543, E/OceanModelEnsemble.py:138-150,
E/MultiLevelOceanEnsemble.py:95-141; E/ = src/gpuocean/ensembles), which
costs (members x kernels) launches per time step.  Here every member - of
any grid size - advances in one persistent launch per RK2 step over a
member/tile work queue, and a block of steps is replayed as one CUDA graph.

Per member the step sequence is exactly that of ``CDKLM16.step(t_end)``
(S/CDKLM16.py:493-509): local_dt = float32(min(dt, float32(t_end - t_now))),
t_now advanced in float64.  Members keep their own dt, so they may take
different numbers of steps; a member whose block is done idles.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .. import _lib
from ..utils import Common


# member grid signature -> index of the fastest tile shape (per process)
_AUTOTUNE_CACHE = {}


class GocMemberDesc(ctypes.Structure):
    """Mirror of ``GocMemberDesc`` in include/gpuocean_gb300.h."""
    _fields_ = [
        ("p", _lib.GocCdklmParams),
        ("Hi", ctypes.c_void_p), ("Hi_pitch", ctypes.c_int32),
        ("Hm", ctypes.c_void_p), ("Hm_pitch", ctypes.c_int32),
        ("eta", ctypes.c_void_p * 2), ("hu", ctypes.c_void_p * 2), ("hv", ctypes.c_void_p * 2),
        ("pitch", ctypes.c_int32),
    ]


def step_schedule(dt, t_end):
    """The dt sequence of one ``step(t_end)`` call (S/CDKLM16.py:493-509)."""
    out = []
    t_now = 0.0
    while t_now < t_end:
        local_dt = np.float32(min(dt, np.float32(t_end - t_now)))
        out.append(local_dt)
        t_now += np.float64(local_dt)
    return out


def step_schedules(dts, t_end, active):
    """step_schedule for many members at once: dts (N,) float32, active
    (N,) bool.  Returns (table (N, K) float32, n (N,) int32), row m holding
    member m's dt sequence - the same numbers step_schedule gives, as every
    member's arithmetic is the same sequence of float32 / float64 roundings."""
    dts = np.asarray(dts, dtype=np.float32)
    t_now = np.zeros(dts.shape[0], dtype=np.float64)
    going = np.array(active, dtype=bool) & (t_now < t_end)
    cols = []
    n = np.zeros(dts.shape[0], dtype=np.int32)
    while going.any():
        local = np.minimum(dts, (t_end - t_now).astype(np.float32))
        cols.append(np.where(going, local, np.float32(0.0)).astype(np.float32))
        n += going
        t_now = np.where(going, t_now + local.astype(np.float64), t_now)
        going &= t_now < t_end
    table = np.stack(cols, axis=1) if cols else np.zeros((dts.shape[0], 0), dtype=np.float32)
    return table, n


class _Schedules:
    """Per-member dt sequences of a block, read from the (table, n) pair."""

    def __init__(self, table, n):
        self.table, self.n = table, n

    def __getitem__(self, m):
        return list(self.table[m, :self.n[m]])

    def __len__(self):
        return len(self.n)


class BatchedEnsemble:
    """Steps a list of RK2 ``CDKLM16`` simulators together on one GPU stream.

    share_bathymetry: point members with identical corner depths (and members
    with identical per-cell Coriolis tables) at one copy
    (None = detect by comparing the device arrays once).
    use_graph: replay each distinct block schedule as a CUDA graph.
    """

    def __init__(self, sims, share_bathymetry=None, use_graph=True, stream=None, autotune=True):
        assert len(sims) > 0
        for s in sims:
            assert int(s.rk_order) == 2, "the batched engine runs the fused RK2 step"
            if getattr(s, "angle_varies", False):
                raise NotImplementedError("a north-angle texture is stepped stage by stage; step such members on "
                                          "their own")
            if s.boundary_conditions.isSponge():
                raise NotImplementedError("sponge boundaries act between the RK stages; step such members on their own")
        self.sims = list(sims)
        self.stream = stream if stream is not None else Common.Stream()
        self.use_graph = use_graph
        self.kernels_launched = 0
        self._graphs = {}
        self._handle = None
        self._noise = None
        self._noise_kind = None
        self._noises = None
        self._noise_sources = None
        self._rng_seed = None
        self._bathy_owner = list(range(len(sims)))
        self._coriolis_owner = list(range(len(sims)))
        self._shape_index = 0
        if share_bathymetry is None:
            share_bathymetry = True
        if share_bathymetry:
            self._dedupe_bathymetry()
            self._dedupe_coriolis()
        self._orig_streams = []
        self._adopt_streams(self.sims)
        self._build()
        if autotune:
            self.autotune()

    # ------------------------------------------------------------------
    def _dedupe_bathymetry(self):
        seen = {}
        for m, s in enumerate(self.sims):
            Bi = np.ma.getdata(s.bathymetry.Bi.download(s.gpu_stream))
            key = (Bi.shape, Bi.tobytes().__hash__(), int(s.boundary_conditions.north), int(s.boundary_conditions.east))
            if key in seen and np.array_equal(seen[key][1], Bi):
                self._bathy_owner[m] = seen[key][0]
            else:
                seen[key] = (m, Bi)

    def _dedupe_coriolis(self):
        # members with identical per-cell Coriolis tables (beta planes) read
        # one copy, which then stays in L2 instead of one copy per member
        seen = {}
        for m, s in enumerate(self.sims):
            if s.coriolis_cell is None:
                continue
            F = np.ascontiguousarray(np.ma.getdata(s.coriolis_cell.download(s.gpu_stream)))
            key = (F.shape, F.tobytes().__hash__())
            if key in seen and np.array_equal(seen[key][1], F):
                self._coriolis_owner[m] = seen[key][0]
            else:
                seen[key] = (m, F)

    def _descs(self):
        descs = (GocMemberDesc * len(self.sims))()
        for m, s in enumerate(self.sims):
            d = descs[m]
            s._params = s._make_params()
            d.p = s._params
            b = self.sims[self._bathy_owner[m]].bathymetry
            d.Hi, d.Hi_pitch = b.Bi.ptr, int(b.Bi.pitch)
            d.Hm, d.Hm_pitch = b.Bm.ptr, int(b.Bm.pitch)
            c = self.sims[self._coriolis_owner[m]].coriolis_cell
            if c is not None:
                d.p.coriolis_cell, d.p.coriolis_cell_pitch = c.ptr, int(c.pitch)
            g = s.gpu_data
            d.eta[0], d.eta[1] = g.h0.ptr, g.h1.ptr
            d.hu[0], d.hu[1] = g.hu0.ptr, g.hu1.ptr
            d.hv[0], d.hv[1] = g.hv0.ptr, g.hv1.ptr
            d.pitch = int(g.h0.pitch)
        return descs

    def _current_ptrs(self):
        return tuple(s.gpu_data.h0.ptr for s in self.sims)

    def _build(self, max_substeps=8):
        self._release_handles()
        self._descs_host = self._descs()
        h = ctypes.c_void_p()
        _lib.call("goc_ensemble_create", self._descs_host, len(self.sims), int(max_substeps), ctypes.byref(h))
        self._handle = h.value
        if self._shape_index:
            _lib.call("goc_ensemble_set_tile_shape", self._handle, int(self._shape_index))
        self.max_substeps = int(max_substeps)
        self._ptrs = self._current_ptrs()
        self._graphs = {}
        self._sched_key = None
        self._mask_key = None
        self._dt_dev = Common.DevicePtr(4 * len(self.sims))
        self._attach_drifters()
        self._collect_streams()
        if getattr(self, "_noises", None) is not None:
            # a rebuilt handle gets new generator states: continue from a new seed
            self._reseeds = getattr(self, "_reseeds", 0) + 1
            seed = None if self._rng_seed is None else self._rng_seed + 7919 * self._reseeds
            self.set_noise(self._noises, getattr(self, "_random_pool", None), rng_seed=seed,
                           sources=self._noise_sources)

    def _adopt_streams(self, objs):
        """Members (and their drifters and model errors) issue their own
        work on the engine's stream while they belong to the engine, so a
        member's calls (download, upload, perturbState, ...) and the
        engine's launches are ordered without any synchronisation.  The
        original streams come back with release()."""
        for s in objs:
            s.gpu_stream.synchronize()
            for o in (s, getattr(s, "drifters", None) if getattr(s, "hasDrifters", False) else None,
                      getattr(s, "model_error", None)):
                if o is None or getattr(o, "gpu_stream", None) is self.stream:
                    continue
                self._orig_streams.append((o, o.gpu_stream))
                o.gpu_stream = self.stream
                rng = getattr(o, "rng", None)
                if rng is not None and hasattr(rng, "gpu_stream"):
                    self._orig_streams.append((rng, rng.gpu_stream))
                    rng.gpu_stream = self.stream

    def _restore_streams(self):
        self.stream.synchronize()
        for o, st in reversed(getattr(self, "_orig_streams", [])):
            o.gpu_stream = st
        self._orig_streams = []

    def _collect_streams(self):
        """The members' own streams (simulator, drifters, model error): the
        engine's stream is ordered after them before it reads the members
        and they after it once it has written them, on the device, so a
        member's own calls (download, upload, perturbState, ...) always see
        the engine's results and the engine theirs."""
        handles = {}
        for s in self.sims:
            objs = [s.gpu_stream]
            if s.hasDrifters:
                objs.append(getattr(s.drifters, "gpu_stream", None))
            if getattr(s, "model_error", None) is not None:
                objs.append(getattr(s.model_error, "gpu_stream", None))
            for o in objs:
                h = Common._stream_handle(o)
                if h is not None and h != self.stream.handle:
                    handles[h] = None
        self._member_streams = (ctypes.c_void_p * max(1, len(handles)))(*handles.keys())
        self._n_member_streams = len(handles)

    def _after_members(self):
        """Engine stream waits for the work queued on the members' streams
        (those not adopted: none unless a member's objects were replaced)."""
        if self._n_member_streams:
            _lib.call("goc_stream_fan_in", self.stream.handle, self._member_streams, self._n_member_streams)

    def _before_members(self):
        """Members' streams wait for the work queued on the engine stream."""
        if self._n_member_streams:
            _lib.call("goc_stream_fan_out", self.stream.handle, self._member_streams, self._n_member_streams)

    def _attach_drifters(self):
        """Drifter collections attached to the members are advected inside
        the batched step; those with wind drift in launches of their own,
        with the collection's wind textures."""
        ptrs = (ctypes.c_void_p * len(self.sims))()
        counts = np.zeros(len(self.sims), dtype=np.int32)
        winds = (_lib.GocDriftWindDesc * len(self.sims))()
        sens = 1.0
        self.has_drifters = False
        self._wind_members = []
        for m, s in enumerate(self.sims):
            d = s.drifters if s.hasDrifters else None
            if d is not None and hasattr(d, "driftersDevice"):
                ptrs[m] = d.driftersDevice.ptr
                counts[m] = d.getNumDrifters()
                sens = d.sensitivity
                self.has_drifters = True
                if d.wind_drift_factor:
                    w = winds[m]
                    w.x_current, w.x_next = d.wind_x_current_arr.ptr, d.wind_x_next_arr.ptr
                    w.y_current, w.y_next = d.wind_y_current_arr.ptr, d.wind_y_next_arr.ptr
                    w.nx, w.ny = int(d.wind_x_current_arr.nx_halo), int(d.wind_x_current_arr.ny_halo)
                    w.wind_drift_factor = float(d.wind_drift_factor)
                    self._wind_members.append(m)
        if self.has_drifters:
            _lib.call("goc_ensemble_set_drifters", self._handle, ptrs, counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      ctypes.c_float(sens), self.stream.handle)
        if self._wind_members:
            _lib.call("goc_ensemble_set_drift_wind", self._handle, winds, self.stream.handle)

    def _wind_times(self, scheds):
        """Time weights of the wind textures for every drift of the block
        (the drift after step k reads the wind at the member's time before
        step k's increment, D/GPUDrifterCollection.py:138-174), after
        bringing each collection's current/next textures to the block's wind
        interval.  A block may not cross a wind time stamp; it may start or
        end on one (the wind there is the same from either side)."""
        table = np.zeros((len(self.sims), self.max_substeps), dtype=np.float32)
        for m in self._wind_members:
            s = self.sims[m]
            d = s.drifters
            t = float(s.t)
            times = []
            for local_dt in scheds[m]:
                times.append(t)
                t += float(np.float64(local_dt))
            if not times:
                continue
            common = None
            for x in times:
                c = {d.wind_interval(x, "left"), d.wind_interval(x, "right")}
                common = c if common is None else common & c
            if not common:
                raise NotImplementedError("a batched block crosses a wind time stamp of member %d's drifters: "
                                          "step to the time stamp first" % m)
            t0, t1 = min(common)
            d.load_wind_interval(t0, t1)
            for k, x in enumerate(times):
                table[m, k] = np.float32(d.wind_weight(x, t0, t1))
        _lib.call("goc_ensemble_set_wind_times", self._handle, table.ctypes.data, self.stream.handle)

    def release(self):
        """Free the device handles and give the members their own streams back."""
        self._release_handles()
        self._restore_streams()

    def _release_handles(self):
        self.release_noise()
        for name in ("_obs_pos", "_obs_out", "_drift_gather", "_obs_scatter"):
            buf = getattr(self, name, None)
            if buf is not None:
                buf.free()
                setattr(self, name, None)
        for g in getattr(self, "_graphs", {}).values():
            _lib.load().goc_graph_destroy(g[0])
        self._graphs = {}
        if getattr(self, "_handle", None):
            _lib.load().goc_ensemble_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @property
    def n_tiles(self):
        nm, nt = ctypes.c_int(), ctypes.c_int()
        _lib.call("goc_ensemble_size", self._handle, ctypes.byref(nm), ctypes.byref(nt))
        return nt.value

    def _check_staging(self):
        """Raise if a block that has completed on the device lost a CTA to a
        TMA copy of its input that never landed (the device flag, copied to
        host memory at the end of every block; no synchronisation)."""
        errors = ctypes.c_int()
        _lib.call("goc_ensemble_staging_errors", self._handle, ctypes.byref(errors))
        if errors.value:
            raise RuntimeError("batched step: a TMA staging wait ran out; the ensemble state is not valid")

    def tma_status(self):
        """(members whose interior tiles stage their input state by TMA,
        tiles staged so far, staging waits that ran out - 0 in normal
        operation).  Synchronises."""
        staged, tiles, errors = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
        _lib.call("goc_ensemble_tma_status", self._handle, ctypes.byref(staged), ctypes.byref(tiles),
                  ctypes.byref(errors))
        return staged.value, tiles.value, errors.value

    # ------------------------------------------------------------------
    @staticmethod
    def tile_shapes():
        """The output tile shapes (cells) the persistent kernel can run."""
        lib = _lib.load()
        out = []
        for i in range(lib.goc_ensemble_tile_shape_count()):
            tx, ty = ctypes.c_int(), ctypes.c_int()
            _lib.call("goc_ensemble_tile_shape", i, ctypes.byref(tx), ctypes.byref(ty))
            out.append((tx.value, ty.value))
        return out

    @property
    def tile_shape(self):
        return self.tile_shapes()[self._shape_index]

    def set_tile_shape(self, index):
        _lib.call("goc_ensemble_set_tile_shape", self._handle, int(index))
        self._shape_index = int(index)
        for g in self._graphs.values():
            _lib.load().goc_graph_destroy(g[0])
        self._graphs = {}

    def _grid_signature(self):
        sizes = {}
        for s in self.sims:
            key = (int(s.nx), int(s.ny))
            sizes[key] = sizes.get(key, 0) + 1
        flags = tuple(sorted({(s.coriolis_cell is None, int(s.boundary_conditions.east)) for s in self.sims}))
        return (tuple(sorted(sizes.items())), flags)

    def autotune(self, repeats=5, candidates=None):
        """Time the persistent RK2 launch of every tile shape on this
        ensemble and keep the fastest.  Each timed launch is RK2 step 0 of a
        one-step schedule: it reads buffer set 0 (the current state) and
        writes set 1, so the members' state is left as it was.  Results are
        cached per process by member grid sizes."""
        sig = self._grid_signature()
        best = _AUTOTUNE_CACHE.get(sig)
        if best is None:
            self._after_members()
            shapes = self.tile_shapes()
            idx = list(range(len(shapes))) if candidates is None else list(candidates)
            n = len(self.sims)
            table = np.zeros((n, self.max_substeps), dtype=np.float32)
            table[:, 0] = [np.float32(s.dt) for s in self.sims]
            nsub = np.ones(n, dtype=np.int32)
            _lib.call("goc_ensemble_set_schedule", self._handle, table.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                      nsub.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), self.stream.handle)
            self._sched_key = None
            ev = [ctypes.c_void_p(), ctypes.c_void_p()]
            for e in ev:
                _lib.call("goc_event_create", ctypes.byref(e))
            timings = {}
            for i in idx:
                _lib.call("goc_ensemble_set_tile_shape", self._handle, int(i))
                for _ in range(2):
                    _lib.call("goc_ensemble_rk2_substep", self._handle, 0, self.stream.handle)
                _lib.call("goc_event_record", ev[0], self.stream.handle)
                for _ in range(repeats):
                    _lib.call("goc_ensemble_rk2_substep", self._handle, 0, self.stream.handle)
                _lib.call("goc_event_record", ev[1], self.stream.handle)
                self.stream.synchronize()
                ms = ctypes.c_float()
                _lib.call("goc_event_elapsed_ms", ev[0], ev[1], ctypes.byref(ms))
                timings[shapes[i]] = ms.value / repeats
            for e in ev:
                _lib.load().goc_event_destroy(e)
            best = min(idx, key=lambda i: timings[shapes[i]])
            _AUTOTUNE_CACHE[sig] = best
            self.autotune_timings = timings
        self.set_tile_shape(best)
        return self.tile_shape

    # ------------------------------------------------------------------
    def _schedule(self, t_end, members=None):
        """Per member the dt sequence of step(t_end); members not in
        `members` (if given) take no step."""
        active = np.ones(len(self.sims), dtype=bool)
        if members is not None:
            active[:] = False
            active[[int(m) for m in members]] = True
        dts = np.fromiter((s.dt for s in self.sims), dtype=np.float32, count=len(self.sims))
        part, n = step_schedules(dts, float(t_end), active)
        nsub = int(n.max()) if len(n) else 0
        if nsub > self.max_substeps or self._current_ptrs() != self._ptrs:
            # members stepped on their own, or a longer block: rebuild the table
            self._build(max_substeps=max(nsub, self.max_substeps))
        table = np.zeros((len(self.sims), self.max_substeps), dtype=np.float32)
        table[:, :part.shape[1]] = part
        return _Schedules(table, n), table, n, nsub

    # ------------------------------------------------------------------
    def set_noise(self, noises, random_pool=None, rng_seed=None, sources=None):
        """Model error of every member in two launches per perturbation.

        noises: one OceanStateNoise (SOAR) or one ModelErrorKL per member.
        random_pool (SOAR): optional device array holding every member's
        random field back to back (one upload refreshes them all); by default
        each member's own buffer is used.  rng_seed: draw fresh XORWOW normals
        on the device before every perturbation (otherwise the random fields
        are used as they are, e.g. injected from the host).  sources (KL):
        sources[m] is the member whose normals and rollers member m uses -
        drawn on the device with the normals when rng_seed is given, else
        from each member's own generator on the host, as perturbSim does -
        the coarse partner of a multi-level pair perturbed "similar as" its
        fine partner (S/CDKLM16.py:782-790); by default every member its own.
        """
        from ..SWEsimulators.ModelErrorKL import GocKLDesc, ModelErrorKL
        assert len(noises) == len(self.sims)
        self.release_noise()
        for n in noises:
            if getattr(n, "gpu_stream", None) is not self.stream:
                n.gpu_stream.synchronize()
                self._orig_streams.append((n, n.gpu_stream))
                n.gpu_stream = self.stream
                rng = getattr(n, "rng", None)
                if rng is not None and hasattr(rng, "gpu_stream"):
                    self._orig_streams.append((rng, rng.gpu_stream))
                    rng.gpu_stream = self.stream
        if all(isinstance(n, ModelErrorKL) for n in noises):
            src = np.arange(len(self.sims), dtype=np.int32) if sources is None else \
                np.ascontiguousarray(sources, dtype=np.int32)
            descs = (GocKLDesc * len(self.sims))(*[n.batch_descriptor(s) for n, s in zip(noises, self.sims)])
            h = ctypes.c_void_p()
            _lib.call("goc_kl_batch_create", self._handle, descs, src.ctypes.data, int(self.max_substeps) + 1,
                      ctypes.byref(h))
            self._noise, self._noise_kind = h.value, "kl"
            self._noise_sources = src
            self._kl_rollers = np.zeros((int(self.max_substeps) + 1, len(self.sims), 4), dtype=np.float32)
            if rng_seed is not None:
                _lib.call("goc_kl_batch_seed", self._noise, ctypes.c_ulonglong(int(rng_seed)), self.stream.handle)
            else:
                # the members' own current normals
                for m, n in enumerate(noises):
                    if src[m] == m:
                        rn = np.ascontiguousarray(n.getRandomNumbers(), dtype=np.float32)
                        _lib.call("goc_kl_batch_set_random", self._noise, m, rn.ctypes.data, self.stream.handle)
                self.stream.synchronize()
        else:
            from ..SWEsimulators.OceanStateNoise import GocNoiseDesc
            descs = (GocNoiseDesc * len(self.sims))()
            off = 0
            for m, (n, s) in enumerate(zip(noises, self.sims)):
                d = n.descriptor(s.f, s.coriolis_beta, s.g)
                if random_pool is not None:
                    d.random = random_pool.ptr + off
                    off += int(n.rand_ny) * int(n.random_numbers.pitch)
                descs[m] = d
            if random_pool is not None:
                assert off <= random_pool.nbytes, "random pool too small"
            self._random_pool = random_pool
            h = ctypes.c_void_p()
            _lib.call("goc_noise_batch_create", self._handle, descs, ctypes.byref(h))
            self._noise, self._noise_kind = h.value, "soar"
            self._noise_descs = descs
            # the unperturbed copies that fused model error at the block
            # cadence needs are allocated here, outside any graph capture
            _lib.call("goc_ensemble_set_block_noise", self._handle, self._noise, 0)
            _lib.call("goc_ensemble_set_block_noise", self._handle, None, -1)
            if rng_seed is not None:
                _lib.call("goc_noise_batch_seed", self._noise, ctypes.c_ulonglong(int(rng_seed)), self.stream.handle)
        self._noises = noises
        self._rng_seed = rng_seed
        self._collect_streams()
        for g in self._graphs.values():
            _lib.load().goc_graph_destroy(g[0])
        self._graphs = {}

    def set_kl_random(self, member, normals):
        """Inject the (2 Ny, Nx) normals that member `member` (and every
        member whose source it is) uses at the next perturbations."""
        assert self._noise_kind == "kl"
        rn = np.ascontiguousarray(normals, dtype=np.float32)
        _lib.call("goc_kl_batch_set_random", self._noise, int(member), rn.ctypes.data, self.stream.handle)
        self.stream.synchronize()

    def _kl_draw_rollers(self, sets):
        """Rollers of the coming perturbations: for every roller set k and
        every source member that perturbs there, four uniforms from its
        model error's generator in the order x_sin, y_sin, x_cos, y_cos, as
        each perturbSim call of the reference draws them
        (S/ModelErrorKL.py:277-300).  sets: list of (set index, members)."""
        r = self._kl_rollers
        for k, members in sets:
            for m in members:
                if self._noise_sources[m] != m:
                    continue
                me = self._noises[m]
                me._setRollers(None, None, None, None)
                r[k, m] = (me.roll_x_sin, me.roll_y_sin, me.roll_x_cos, me.roll_y_cos)
        n_sets = max(k for k, _ in sets) + 1
        _lib.call("goc_kl_batch_set_rollers", self._noise, r.ctypes.data, int(n_sets), self.stream.handle)

    def release_noise(self):
        if getattr(self, "_noise", None):
            if self._noise_kind == "kl":
                _lib.load().goc_kl_batch_destroy(self._noise)
            else:
                _lib.load().goc_noise_batch_destroy(self._noise)
            self._noise = None

    def _noise_launch(self, substep, scale=1.0, update_random_field=True):
        if self._noise_kind == "kl":
            if update_random_field and self._rng_seed is not None:
                _lib.call("goc_kl_batch_generate", self._noise, self._handle, int(substep), self.stream.handle)
            _lib.call("goc_kl_batch_perturb", self._noise, self._handle, ctypes.c_float(scale), int(substep),
                      self.stream.handle)
            return
        if update_random_field and self._rng_seed is not None:
            _lib.call("goc_noise_batch_generate", self._noise, self._handle, int(substep), self.stream.handle)
        _lib.call("goc_noise_batch_perturb", self._noise, self._handle, ctypes.c_float(scale), int(substep),
                  self.stream.handle)

    def perturb(self, perturbation_scale=1.0, update_random_field=True):
        """Add the SOAR model error to every member's current state."""
        before = _lib.load().goc_kernel_launch_count()
        self._after_members()
        if self._noise_kind == "kl" and not (update_random_field and self._rng_seed is not None):
            # injected normals: rollers from the members' own generators, as
            # perturbSim draws them; with device draws they come with the normals
            self._kl_draw_rollers([(0, range(len(self.sims)))])
        self._noise_launch(-1, perturbation_scale, update_random_field)
        self._before_members()
        self.kernels_launched += _lib.load().goc_kernel_launch_count() - before

    def _noise_field(self, substep):
        """New normals (device generator) and the SOAR coarse fields of the
        members that perturb at `substep` (-1: all), ahead of the fused
        step that adds them."""
        if self._rng_seed is not None:
            _lib.call("goc_noise_batch_generate", self._noise, self._handle, int(substep), self.stream.handle)
        _lib.call("goc_noise_batch_field", self._noise, self._handle, ctypes.c_float(1.0), int(substep),
                  self.stream.handle)

    def _launch_block(self, nsub, noise=None, n=None):
        """noise: None, "block" (once after the block) or "step" (after every
        RK2 step of each member, before its drifters move).  SOAR model error
        is fused into the step launches: the coarse fields are computed
        before the first step that perturbs, and each member's perturbation
        is added to the state the step writes.  KL model error runs as its
        own launches after the steps.  n: the members' step counts."""
        before = _lib.load().goc_kernel_launch_count()
        fused = noise is not None and self._noise_kind == "soar"
        first = -1
        if fused:
            _lib.call("goc_ensemble_set_block_noise", self._handle, self._noise, 0 if noise == "block" else 1)
            first = min((int(x) for x in n if x > 0), default=0) - 1 if noise == "block" else -1
        try:
            for k in range(nsub):
                if fused and (noise == "step" or k == first):
                    self._noise_field(k if noise == "step" else -1)
                _lib.call("goc_ensemble_rk2_substep", self._handle, k, self.stream.handle)
                if noise == "step" and not fused:
                    self._noise_launch(k)
            _lib.call("goc_ensemble_end_block", self._handle, int(nsub), self.stream.handle)
        finally:
            if fused:
                _lib.call("goc_ensemble_set_block_noise", self._handle, None, -1)
        if noise == "block" and not fused:
            self._noise_launch(-2)   # the members that take model error in this block
        return _lib.load().goc_kernel_launch_count() - before

    def step(self, t_end, apply_stochastic_term=False, noise_cadence="block", members=None):
        """Advance the members by ``t_end`` seconds (one block).  With
        ``apply_stochastic_term`` the model error is added either once after
        the block (``noise_cadence="block"``, the ``dataAssimilationStep``
        cadence, S/CDKLM16.py:786-790) or after every RK2 step
        (``"step"``, the cadence of ``CDKLM16.step``, S/CDKLM16.py:567-568).
        ``apply_stochastic_term`` may be one flag per member (a truth and
        particles with different flags, E/OceanNoiseEnsemble.py:517-532).
        ``members``: indices of the members to advance (default all); the
        others keep their state and time.  Returns the number of
        member-cell-steps taken."""
        assert noise_cadence in ("block", "step")
        flags = np.broadcast_to(np.asarray(apply_stochastic_term, dtype=bool), (len(self.sims),))
        with_noise = noise_cadence if (flags.any() and getattr(self, "_noise", None) is not None) else None
        chosen = range(len(self.sims)) if members is None else [int(m) for m in members]
        for m in chosen:
            s = self.sims[m]
            if s.t == 0:
                s.bc_kernel.boundaryCondition(s.gpu_stream, s.gpu_data.h0, s.gpu_data.hu0, s.gpu_data.hv0)
        scheds, table, n, nsub = self._schedule(t_end, members)
        self._after_members()
        mask = flags.astype(np.int32)
        if with_noise is not None and mask.tobytes() != getattr(self, "_mask_key", None):
            _lib.call("goc_ensemble_set_noise_mask", self._handle, mask.ctypes.data, self.stream.handle)
            self._mask_key = mask.tobytes()
        if with_noise is not None and self._noise_kind == "kl" and self._rng_seed is None:
            if with_noise == "block":
                self._kl_draw_rollers([(0, [m for m in range(len(self.sims)) if mask[m]])])
            else:
                self._kl_draw_rollers([(k + 1, [m for m in range(len(self.sims)) if n[m] > k and mask[m]])
                                       for k in range(nsub)])
        if getattr(self, "_wind_members", None):
            self._wind_times(scheds)
        key = (n.tobytes(), table.tobytes())
        if key != getattr(self, "_sched_key", None):
            _lib.call("goc_ensemble_set_schedule", self._handle, table.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                      n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), self.stream.handle)
            self._sched_key = key
        if self.use_graph:
            # a fused model error depends on which step ends each member's
            # block: such graphs are kept per step-count pattern
            fused = with_noise is not None and self._noise_kind == "soar"
            gkey = (nsub, with_noise, (n.tobytes(), mask.tobytes()) if fused else None)
            entry = self._graphs.get(gkey)
            if entry is None:
                if len(self._graphs) >= 16:
                    old = next(iter(self._graphs))
                    _lib.load().goc_graph_destroy(self._graphs.pop(old)[0])
                _lib.call("goc_graph_begin_capture", self.stream.handle)
                try:
                    nodes = self._launch_block(nsub, with_noise, n)
                finally:
                    gh = ctypes.c_void_p()
                    _lib.call("goc_graph_end_capture", self.stream.handle, ctypes.byref(gh))
                entry = self._graphs[gkey] = (gh.value, nodes)
            _lib.call("goc_graph_launch", entry[0], self.stream.handle)
            self.kernels_launched += entry[1]
        else:
            self.kernels_launched += self._launch_block(nsub, with_noise, n)
        self._before_members()
        self._check_staging()
        # the members' clocks: each member's dts added one by one in float64,
        # as step does; the drifters' clocks by the sum of the block's dts
        steps = table[:, :nsub].astype(np.float64)
        t = np.fromiter((s.t for s in self.sims), dtype=np.float64, count=len(self.sims))
        dsum = np.zeros(len(self.sims), dtype=np.float64)
        for k in range(nsub):
            on = n > k
            t = np.where(on, t + steps[:, k], t)
            dsum = np.where(on, dsum + steps[:, k], dsum)
        for m in np.flatnonzero(n):
            s = self.sims[m]
            s.t = t[m]
            s.num_iterations += int(n[m])
            if s.hasDrifters:
                s.drifter_t += dsum[m]
            if n[m] % 2 == 1:
                s.gpu_data.swap()
        self._ptrs = self._current_ptrs()
        return int(np.dot(n.astype(np.int64), self._member_cells()))

    def _member_cells(self):
        cells = getattr(self, "_cells_cache", None)
        if cells is None or len(cells) != len(self.sims):
            cells = self._cells_cache = np.array([int(s.nx) * int(s.ny) for s in self.sims], dtype=np.int64)
        return cells

    def synchronize(self):
        self.stream.synchronize()
        self._check_staging()

    # ------------------------------------------------------------------
    # observation operator and ensemble statistics
    # ------------------------------------------------------------------
    def _ensure_table(self):
        """The device member table must point at the current buffers."""
        if self._current_ptrs() != self._ptrs:
            self._build(max_substeps=self.max_substeps)

    def _scratch(self, name, nbytes):
        buf = getattr(self, name, None)
        if buf is None or buf.nbytes < nbytes:
            if buf is not None:
                buf.free()
            buf = Common.DevicePtr(max(int(nbytes), 256))
            setattr(self, name, buf)
        return buf

    def _download(self, buf, shape, dtype=np.float32):
        out = np.empty(shape, dtype=dtype)
        if out.nbytes:
            _lib.call("goc_memcpy_d2h_async", out.ctypes.data, buf.ptr, ctypes.c_size_t(out.nbytes), self.stream.handle)
        self.stream.synchronize()
        return out

    def observe(self, positions=None, first=0, count=None, drifters=None):
        """(eta, hu, hv) of members [first, first + count) at the cells
        holding the given positions, in one launch: an array (count,
        positions, 3).  positions: (D, 2) metres from the south-west
        interior corner (host), or ``drifters``: a GPUDrifterCollection whose
        device positions every member observes (its last row, the
        observation position, is left out), as the reference's GPU path of
        observeParticles does (E/BaseOceanStateEnsemble.py:113-130)."""
        count = len(self.sims) - first if count is None else int(count)
        self._ensure_table()
        self._after_members()
        if drifters is not None:
            _lib.call("goc_stream_fan_in", self.stream.handle,
                      (ctypes.c_void_p * 1)(Common._stream_handle(drifters.gpu_stream)), 1)
            D = int(drifters.getNumDrifters())
            pos_ptr, pitch = drifters.driftersDevice.ptr, int(drifters.driftersDevice.pitch)
        else:
            pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 2)
            D = pos.shape[0]
            buf = self._scratch("_obs_pos", pos.nbytes)
            if pos.nbytes:
                _lib.call("goc_memcpy_h2d_async", buf.ptr, pos.ctypes.data, ctypes.c_size_t(pos.nbytes),
                          self.stream.handle)
            pos_ptr, pitch = buf.ptr, 8
        out = self._scratch("_obs_out", 12 * count * D)
        before = _lib.load().goc_kernel_launch_count()
        _lib.call("goc_ensemble_observe", self._handle, int(first), count, pos_ptr, pitch, ctypes.c_longlong(0), D,
                  out.ptr, self.stream.handle)
        self.kernels_launched += _lib.load().goc_kernel_launch_count() - before
        return self._download(out, (count, D, 3))

    def drifter_rows(self):
        """Rows of all members' drifter arrays (N_m positions and the
        observation row each), the size of download_drifters' result."""
        rows = ctypes.c_longlong()
        _lib.call("goc_ensemble_drifter_rows", self._handle, ctypes.byref(rows))
        return rows.value

    def download_drifters(self, out=None):
        """Every member's drifter rows, member by member, as one (rows, 2)
        float32 array: one gather launch and one copy instead of a download
        per collection.  out: a host array to fill (pinned memory makes the
        copy asynchronous to the host) or its address as an int."""
        self._ensure_table()
        rows = self.drifter_rows()
        buf = self._scratch("_drift_gather", 8 * rows)
        _lib.call("goc_ensemble_gather_drifters", self._handle, buf.ptr, self.stream.handle)
        self.kernels_launched += 1
        if isinstance(out, int):
            _lib.call("goc_memcpy_d2h_async", out, buf.ptr, ctypes.c_size_t(8 * rows), self.stream.handle)
            return None
        if out is None:
            out = np.empty((rows, 2), dtype=np.float32)
        _lib.call("goc_memcpy_d2h_async", out.ctypes.data, buf.ptr, ctypes.c_size_t(8 * rows), self.stream.handle)
        self.stream.synchronize()
        return out

    def upload_observation_positions(self, positions):
        """The observation row of every member with drifters from an
        (n_members, 2) array (or the address of one in host memory): one
        copy and one scatter launch."""
        n = len(self.sims)
        buf = self._scratch("_obs_scatter", 8 * n)
        if isinstance(positions, int):
            _lib.call("goc_memcpy_h2d_async", buf.ptr, positions, ctypes.c_size_t(8 * n), self.stream.handle)
        else:
            pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(n, 2)
            _lib.call("goc_memcpy_h2d_async", buf.ptr, pos.ctypes.data, ctypes.c_size_t(8 * n), self.stream.handle)
            self.stream.synchronize()
        _lib.call("goc_ensemble_scatter_observations", self._handle, buf.ptr, self.stream.handle)
        self.kernels_launched += 1

    def moments(self, first=0, count=None, quantity="state", desingularise=None, ddof=0, mean=True, var=True,
                download=True):
        """Mean and variance over members [first, first + count) (one grid)
        per interior cell, in one pass over HBM.  quantity "state": planes
        (eta, hu, hv); "velocity": (u, v) = (hu, hv) / (eta + Hm),
        desingularised with eps = ``desingularise`` when given
        (U/OceanographicUtilities.py:413-414).  Returns (mean, var) arrays of
        shape (planes, ny, nx) (None for the one not asked for); with
        ``download=False`` the device buffers instead."""
        count = len(self.sims) - first if count is None else int(count)
        assert quantity in ("state", "velocity")
        self._ensure_table()
        self._after_members()
        s0 = self.sims[first]
        planes = 3 if quantity == "state" else 2
        nbytes = 4 * planes * int(s0.nx) * int(s0.ny)
        bm = Common.DevicePtr(nbytes) if mean else None
        bv = Common.DevicePtr(nbytes) if var else None
        eps = 0.0 if desingularise is None else float(desingularise)
        before = _lib.load().goc_kernel_launch_count()
        _lib.call("goc_ensemble_moments", self._handle, int(first), count, 0 if quantity == "state" else 1,
                  ctypes.c_float(eps), int(ddof), bm.ptr if bm else None, bv.ptr if bv else None, self.stream.handle)
        self.kernels_launched += _lib.load().goc_kernel_launch_count() - before
        if not download:
            return bm, bv
        shape = (planes, int(s0.ny), int(s0.nx))
        out = []
        for b in (bm, bv):
            if b is None:
                out.append(None)
            else:
                out.append(self._download(b, shape))
                b.free()
        return tuple(out)

    def max_dt(self):
        """Per member the CFL limit 0.25 min(dx / |u +- c|, dy / |v +- c|)
        over its interior cells, before the Courant factor (one reduction
        launch pair; synchronises)."""
        self._ensure_table()
        self._after_members()
        _lib.call("goc_ensemble_max_dt", self._handle, self._dt_dev.ptr, self.stream.handle)
        out = np.zeros(len(self.sims), dtype=np.float32)
        _lib.call("goc_memcpy_d2h_async", out.ctypes.data, self._dt_dev.ptr, ctypes.c_size_t(out.nbytes),
                  self.stream.handle)
        self.stream.synchronize()
        return out

    def updateDt(self, courant_number=None, members=None):
        """Batched CFL limit of every member (one reduction launch pair);
        ``members``: indices of the members whose dt is set (default all)."""
        self._after_members()
        _lib.call("goc_ensemble_max_dt", self._handle, self._dt_dev.ptr, self.stream.handle)
        out = np.zeros(len(self.sims), dtype=np.float32)
        _lib.call("goc_memcpy_d2h_async", out.ctypes.data, self._dt_dev.ptr, ctypes.c_size_t(out.nbytes),
                  self.stream.handle)
        self.stream.synchronize()
        chosen = range(len(self.sims)) if members is None else members
        for m in chosen:
            s = self.sims[m]
            cn = s.courant_number if courant_number is None else courant_number
            s.dt = cn * out[m]
        return out


def _main(argv=None):
    """``python -m gpuocean_gb300.ensembles.BatchedEnsemble [--members M]
    [--nx NX] [--ny NY] [--repeats R]``: M members of the double-jet case on
    an NX x NY grid stepped one 60 s block, then R launches each of the
    member moments of (eta, hu, hv) and of one observation of every member
    at 1000 positions; prints their mean times.  A small, self-contained
    workload for timing and profiling the statistics kernels."""
    import argparse
    import json
    from ..SWEsimulators import CDKLM16
    from ..utils import BenchmarkCases
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=128)
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=300)
    ap.add_argument("--repeats", type=int, default=5)
    a = ap.parse_args(argv)
    ctx = Common.CUDAContext()
    c = BenchmarkCases.double_jet_case(nx=a.nx, ny=a.ny, dx=5000.0, dy=5000.0, seed=2)
    b = Common.BoundaryConditions(1, 2, 1, 2)
    sims = [CDKLM16.CDKLM16(ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], a.nx, a.ny, c["dx"], c["dy"], 0.0, c["g"],
                            c["f"], 0.0, coriolis_beta=c["coriolis_beta"], boundary_conditions=b)
            for _ in range(a.members)]
    ens = BatchedEnsemble(sims, autotune=False)
    ens.step(60.0)
    m, v = ens.moments(download=False)
    rng = np.random.default_rng(0)
    pos = np.stack([rng.uniform(0, a.nx * c["dx"], 1000), rng.uniform(0, a.ny * c["dy"], 1000)], axis=1)
    ens.observe(pos)
    ev = [ctypes.c_void_p() for _ in range(3)]
    for e in ev:
        _lib.call("goc_event_create", ctypes.byref(e))
    st = ens.stream.handle
    _lib.call("goc_event_record", ev[0], st)
    for _ in range(a.repeats):
        _lib.call("goc_ensemble_moments", ens._handle, 0, a.members, 0, ctypes.c_float(0.0), 0, m.ptr, v.ptr, st)
    _lib.call("goc_event_record", ev[1], st)
    for _ in range(a.repeats):
        _lib.call("goc_ensemble_observe", ens._handle, 0, a.members, ens._obs_pos.ptr, 8, ctypes.c_longlong(0), 1000,
                  ens._obs_out.ptr, st)
    _lib.call("goc_event_record", ev[2], st)
    ens.synchronize()
    t = [ctypes.c_float(), ctypes.c_float()]
    _lib.call("goc_event_elapsed_ms", ev[0], ev[1], ctypes.byref(t[0]))
    _lib.call("goc_event_elapsed_ms", ev[1], ev[2], ctypes.byref(t[1]))
    cells = a.members * a.nx * a.ny
    print(json.dumps({"members": a.members, "nx": a.nx, "ny": a.ny, "moments_ms": t[0].value / a.repeats,
                      "moments_gbs": (12 * cells + 24 * a.nx * a.ny) / (t[0].value / a.repeats * 1e-3) / 1e9,
                      "observe_ms": t[1].value / a.repeats}))
    for e in ev:
        _lib.load().goc_event_destroy(e)
    m.free()
    v.free()
    ens.release()


if __name__ == "__main__":
    _main()
