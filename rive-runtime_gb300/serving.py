"""Serving loop: animated sessions rendered with continuous batching.

A session's content is either real (RecordedAnimation: the frames of one of the
reference's recorded .riv animations, converted by sriv.py) or synthetic
(AnimatedScene). A synthetic session is one scene (a rive_scene.h recording)
animated on the host:
every transform rotates at its own angular rate and every control point of a
path moves by amplitude * sin(2 pi f t + phi) along a per-path direction. A
session asks for frames at a fixed rate from its arrival on (frame k is due
at arrival + k / fps). For each frame the host turns the session's frame
recording into flush records with the front end the caller supplies (in a
deployment, rive-runtime's own RiveRenderer -> RenderContext through
RenderContextCUDAImpl; in the benchmark and the tests, a stand-in), and the
frame joins the next batch.

Continuous batching: each batch takes every frame that is due (one per
session at most, up to max_batch), so sessions join and leave the batch
composition frame by frame. The records of all frames of a batch are packed
into one device-resident arena per record kind (two arenas, alternating, so
the next batch's upload never overwrites records the GPU may still read), and
the batch renders with one rive_cuda_flush_batch per logical-flush index.
While the GPU renders a batch, the host plans the next one. Sessions are
admitted while their device footprint fits the HBM budget; later arrivals
wait. Frame latency = completion time of the frame's batch on the device
minus the frame's due time.

The reference has no server; its closest analogue is an application calling
Artboard::advance then RenderContext::flush once per frame
(renderer/src/render_context.cpp:770-1044).
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import struct
import time
from dataclasses import dataclass, field

import numpy as np

from .capture import BUFFER_NAMES
from .scene import CMD_TRANSFORM, MAGIC, Scene

HEADER = struct.Struct("<12I")
PATH_REC = 20
PAINT_REC = 56
CMD_REC = 36
ALIGN = 256


class AnimatedScene:
    """A scene whose frames differ only in control points and transforms; a
    frame is the base recording with those two arrays rewritten."""

    def __init__(self, sc: Scene, rng, amplitude: float = 3.0,
                 rate_range=(-math.pi, math.pi), freq_range=(0.2, 2.0)):
        self.width, self.height = sc.width, sc.height
        self.base = bytes(sc.to_bytes())
        h = HEADER.unpack_from(self.base, 0)
        assert h[0] == MAGIC
        npaths, npaints, ncmds, nverbs, npts = h[4], h[5], h[6], h[7], h[8]
        path_off = HEADER.size
        self.cmd_off = path_off + PATH_REC * npaths + PAINT_REC * npaints
        self.pts_off = self.cmd_off + CMD_REC * ncmds + ((nverbs + 3) & ~3)
        self.npts = npts
        self.base_pts = np.frombuffer(self.base, "<f4", 2 * npts, self.pts_off).reshape(-1, 2)
        recs = np.frombuffer(self.base, "<u4", 5 * npaths, path_off).reshape(-1, 5)
        owner = np.zeros(npts, np.int64)
        for i, (_, _, p0, pn, _) in enumerate(recs):
            owner[p0:p0 + pn] = i
        self.owner = owner
        self.freq = rng.uniform(*freq_range, npaths)
        self.phase = rng.uniform(0.0, 2.0 * math.pi, npaths)
        ang = rng.uniform(0.0, 2.0 * math.pi, npaths)
        self.dir = np.stack([np.cos(ang), np.sin(ang)], 1)
        self.amplitude = amplitude
        cmds = np.frombuffer(self.base, "<u4", 9 * ncmds, self.cmd_off).reshape(-1, 9)
        self.tf_idx = np.nonzero(cmds[:, 0] == CMD_TRANSFORM)[0]
        self.tf_base = cmds[self.tf_idx, 3:9].copy().view("<f4").astype(np.float64)
        self.rate = rng.uniform(*rate_range, len(self.tf_idx))

    def frame(self, t: float) -> bytes:
        buf = bytearray(self.base)
        d = self.amplitude * np.sin(2.0 * math.pi * self.freq * t + self.phase)
        pts = (self.base_pts + (d[:, None] * self.dir)[self.owner]).astype("<f4")
        buf[self.pts_off:self.pts_off + 8 * self.npts] = pts.tobytes()
        if len(self.tf_idx):
            th = self.rate * t
            c, s = np.cos(th), np.sin(th)
            a, b, cc, dd, tx, ty = (self.tf_base[:, k] for k in range(6))
            # M * R(theta): the path turns about its own local origin.
            m = np.stack([a * c + cc * s, b * c + dd * s, cc * c - a * s, dd * c - b * s,
                          tx, ty], 1).astype("<f4")
            cm = np.frombuffer(buf, "<u4", len(buf) // 4 - self.cmd_off // 4,
                               self.cmd_off).reshape(-1)
            for j, ci in enumerate(self.tf_idx):
                w = 9 * int(ci) + 3
                cm[w:w + 6] = m[j].view("<u4")
            del cm
        return bytes(buf)


class RecordedAnimation:
    """Real content: the frames of a recorded animation (scene recordings, as
    sriv.unpack_frames returns them), played at `rate` frames per second of
    session time and looped. Frame t is the recording nearest below t."""

    def __init__(self, frames, rate: float = 60.0, offset: int = 0):
        if not frames:
            raise ValueError("an animation needs at least one frame")
        self.frames = list(frames)
        self.rate = rate
        self.offset = offset
        h = HEADER.unpack_from(self.frames[0], 0)
        assert h[0] == MAGIC
        self.width, self.height = h[1], h[2]

    def frame(self, t: float) -> bytes:
        k = int(math.floor(t * self.rate + 1e-6)) + self.offset
        return self.frames[k % len(self.frames)]


@dataclass
class Session:
    sid: int
    anim: AnimatedScene
    frames: int
    fps: float = 60.0
    arrival: float = 0.0
    admitted: float = -1.0
    next_frame: int = 0
    target: object = None
    footprint: int = 0
    latencies: list = field(default_factory=list)

    def due(self, k: int) -> float:
        return self.arrival + k / self.fps


class RecordArenas:
    """Two device arenas per record kind (alternating per batch) and their
    pinned host staging; a batch's records are packed session after session,
    each at a 256-byte boundary."""

    def __init__(self, torch, device):
        self.torch = torch
        self.device = device
        self.slot = 0
        self.host = [dict(), dict()]
        self.dev = [dict(), dict()]

    def _ensure(self, d, name, nbytes, pinned):
        t = d.get(name)
        if t is None or t.numel() < nbytes:
            n = max(int(nbytes * 1.25) + ALIGN, 1 << 16)
            if pinned:
                t = self.torch.empty(n, dtype=self.torch.uint8).pin_memory()
            else:
                t = self.torch.empty(n, dtype=self.torch.uint8, device=f"cuda:{self.device}")
            d[name] = t
        return t

    def pack(self, caps, stream):
        """Copies the batch's records to the device; returns per-capture
        {name: device address} maps."""
        slot = self.slot
        self.slot ^= 1
        offs = [dict() for _ in caps]
        for name in BUFFER_NAMES:
            total = 0
            for i, cap in enumerate(caps):
                n = len(cap.buffers.get(name, b""))
                offs[i][name] = (total, n)
                total += (n + ALIGN - 1) // ALIGN * ALIGN
            if total == 0:
                for i in range(len(caps)):
                    offs[i][name] = None
                continue
            h = self._ensure(self.host[slot], name, total, True)
            d = self._ensure(self.dev[slot], name, total, False)
            hn = h.numpy()
            for i, cap in enumerate(caps):
                o, n = offs[i][name]
                if n:
                    hn[o:o + n] = np.frombuffer(cap.buffers[name], np.uint8)
            with self.torch.cuda.stream(stream):
                d[:total].copy_(h[:total], non_blocking=True)
            base = d.data_ptr()
            for i in range(len(caps)):
                o, n = offs[i][name]
                offs[i][name] = base + o if n else None
        return offs


class FrameServer:
    """Continuous-batching frame server on one rive_cuda context.

    `front_end(frame_bytes) -> capture.Capture` turns one frame recording of a
    session into its flush records; it runs on `planner_threads` host threads
    (it must release the GIL to overlap)."""

    def __init__(self, ctx, front_end, device: int = 0, hbm_budget_bytes: int = 120 << 30,
                 max_batch: int = 256, planner_threads: int = 8, keep_frames=()):
        import torch
        self.torch = torch
        self.front_end = front_end
        self.ctx = ctx
        self.device = device
        self.budget = hbm_budget_bytes
        self.max_batch = max_batch
        self.pool = cf.ThreadPoolExecutor(planner_threads)
        self.stream = torch.cuda.Stream(device)
        self.arenas = RecordArenas(torch, device)
        self.active: list[Session] = []
        self.waiting: list[Session] = []
        self.finished: list[Session] = []
        self.reserved = 0
        self.peak_reserved = 0
        self.batches = 0
        self.frames = 0
        self.max_concurrent = 0
        self.keep = set(keep_frames)   # (sid, frame) whose images are kept
        self.kept = {}

    @staticmethod
    def footprint(cap) -> int:
        """Device bytes a session holds while active: its target, twice its
        records (two arenas) and its share of the intermediates."""
        rec = sum(len(cap.buffers.get(n, b"")) for n in BUFFER_NAMES)
        verts = sum(max(f.desc["tess_data_height"], 1) for f in cap.flushes) * 2048
        slots = sum(int(f.batches[:, 1].sum()) for f in cap.flushes if len(f.batches)) * 24
        return int(cap.width * cap.height * 4 + 2 * 1.25 * rec + verts * 16 + slots * (96 + 8)
                   + slots * 4 * 16)

    def _plan(self, s: Session, k: int):
        return self.front_end(s.anim.frame(k / s.fps))

    def _admit(self, now):
        still = []
        for s in self.waiting:
            cap0 = self._plan(s, 0)
            need = self.footprint(cap0)
            if self.reserved + need > self.budget and self.active:
                still.append(s)
                continue
            s.footprint = need
            s.admitted = now
            self.reserved += need
            self.peak_reserved = max(self.peak_reserved, self.reserved)
            s.target = self.torch.zeros((cap0.height, cap0.width, 4), dtype=self.torch.uint8,
                                        device=f"cuda:{self.device}")
            self.active.append(s)
        self.waiting = still
        self.max_concurrent = max(self.max_concurrent, len(self.active))

    def run(self, sessions, timeout_s: float = 600.0):
        """Serves `sessions` (arrival times in seconds from the start) until
        every one has rendered all its frames; returns the statistics."""
        pending = sorted(sessions, key=lambda s: s.arrival)
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        # Device-side completion times: a timing event at the start of the
        # run (the stream is idle, so it completes at once) is the origin.
        self.ev0 = self.torch.cuda.Event(enable_timing=True)
        self.ev0.record(self.stream)
        self.ev0.synchronize()
        self.t_ev0 = clock()
        inflight = None
        planned = None  # (sessions, frame indices, caps) for the next batch
        while pending or self.waiting or self.active or inflight:
            now = clock()
            if now > timeout_s:
                raise TimeoutError("serving loop exceeded its time limit")
            while pending and pending[0].arrival <= now:
                self.waiting.append(pending.pop(0))
            if self.waiting:
                self._admit(now)
            if planned is None:
                # Frames due now, one per session, earliest first.
                cand = [s for s in self.active if s.next_frame < s.frames
                        and s.due(s.next_frame) <= now]
                cand.sort(key=lambda s: s.due(s.next_frame))
                cand = cand[:self.max_batch]
                if cand:
                    ks = [s.next_frame for s in cand]
                    for s in cand:
                        s.next_frame += 1
                    caps = list(self.pool.map(lambda sk: self._plan(*sk), zip(cand, ks)))
                    planned = (cand, ks, caps)
            if inflight is not None:
                self._retire(inflight, clock)
                inflight = None
            if planned is not None:
                inflight = self._submit(*planned)
                planned = None
            elif not pending and not self.waiting and not self.active:
                break
            else:
                # Nothing due yet: sleep until the next due frame or arrival.
                nxt = [s.due(s.next_frame) for s in self.active if s.next_frame < s.frames]
                if pending:
                    nxt.append(pending[0].arrival)
                if nxt:
                    time.sleep(max(0.0, min(min(nxt) - clock(), 0.002)))
        self.pool.shutdown(wait=True)
        wall = clock()
        lat = np.array([x for s in self.finished for x in s.latencies]) * 1e3
        return {
            "sessions": len(self.finished), "frames": int(self.frames), "batches": self.batches,
            "wall_s": wall, "frames_per_s": self.frames / wall if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_batch": self.frames / max(self.batches, 1),
            "max_concurrent": self.max_concurrent,
            "peak_reserved_gb": self.peak_reserved / 2**30,
        }

    def _submit(self, sessions, ks, caps):
        from .rive_cuda import DeviceBuffers
        addrs = self.arenas.pack(caps, self.stream)
        waves = max(len(c.flushes) for c in caps)
        for w in range(waves):
            items = []
            for s, c, a in zip(sessions, caps, addrs):
                if w < len(c.flushes):
                    b = DeviceBuffers()
                    for name in BUFFER_NAMES:
                        setattr(b, name, a[name])
                    items.append((c.flushes[w], b, s.target.data_ptr()))
            self.ctx.flush_batch(items, self.stream.cuda_stream)
        ev = self.torch.cuda.Event(enable_timing=True)
        ev.record(self.stream)
        self.batches += 1
        return (sessions, ks, ev)

    def _retire(self, inflight, clock):
        sessions, ks, ev = inflight
        ev.synchronize()
        self.ctx.sync(self.stream.cuda_stream)
        t = self.t_ev0 + self.ev0.elapsed_time(ev) * 1e-3  # when the batch finished
        for s, k in zip(sessions, ks):
            s.latencies.append(t - s.due(k))
            if (s.sid, k) in self.keep:
                self.kept[(s.sid, k)] = s.target.cpu().numpy().copy()
            self.frames += 1
            if k + 1 >= s.frames:
                self.active.remove(s)
                self.finished.append(s)
                self.reserved -= s.footprint
                s.target = None


def poisson_sessions(scenes, rate_per_s: float, frames: int, fps: float = 60.0, seed: int = 0):
    """Sessions over `scenes`, arriving by a Poisson process of `rate_per_s`."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i, sc in enumerate(scenes):
        t += rng.exponential(1.0 / rate_per_s)
        out.append(Session(sid=i, anim=AnimatedScene(sc, rng), frames=frames, fps=fps, arrival=t))
    return out


def recorded_sessions(animations, count: int, rate_per_s: float, frames: int,
                      fps: float = 60.0, seed: int = 0):
    """`count` sessions, each playing one of `animations` (lists of frame
    recordings, in turn) from a random start frame, arriving by a Poisson
    process of `rate_per_s`."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate_per_s)
        fr = animations[i % len(animations)]
        anim = RecordedAnimation(fr, rate=fps, offset=int(rng.integers(len(fr))))
        out.append(Session(sid=i, anim=anim, frames=frames, fps=fps, arrival=t))
    return out


def render_alone(ctx, front_end, s: Session, k: int, stream=None):
    """Frame k of session s rendered by itself (one flush at a time), for the
    alone-versus-in-the-mix check."""
    import torch
    from .rive_cuda import DeviceBuffers
    cap = front_end(s.anim.frame(k / s.fps))
    keep = []
    b = DeviceBuffers()
    for name in BUFFER_NAMES:
        data = cap.buffers.get(name, b"")
        t = torch.from_numpy(np.frombuffer(data, np.uint8).copy()).cuda() if data else None
        keep.append(t)
        setattr(b, name, t.data_ptr() if t is not None else None)
    out = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")
    for f in cap.flushes:
        ctx.flush_device(f, b, out.data_ptr(), stream)
    ctx.sync(stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()
