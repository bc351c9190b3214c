"""The online input path on the GPU: detector-module packets -> assembled ring
frames -> the batched engine, against the FP64 oracle on the same frames.

One Python thread per detector module (27 modules of 16 detectors, 500
projections, 10 projections per packet, 50 parts per module and frame) feeds
its packets through risa_gb_assembler_ingest (ctypes releases the GIL, so the
module threads run concurrently) into a pinned ring of module-major frames.
The consumer takes each handed-out frame, copies it from its ring slot to the
device and releases the slot; the frames then run through risa_gb_fbp_enqueue
with module_major set, and every image is compared with the oracle's
reconstruction of the very bytes that were handed out (converted to
detector-major order), at max-rel 1e-5 and rel-L2 1e-5.

  exact rule: packets of two consecutive frames shuffled per module, one
    packet lost, so that frame is given up once a frame skip_lag newer is
    complete; every other frame arrives, bit-identical to what was sent.
  last_part rule (the reference's OnlineReceiverNotification): parts in order
    per module, one middle part lost; frame 0 is never handed out, the frame
    with the lost part is handed out with that part's region holding what its
    slot held before, and the indices handed out increase.
"""
import random
import threading
import time

import numpy as np
import pytest

import oracle
import risa_gb300 as rg
from risa_gb300 import phantom
from tests.helpers import ns, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_REL = 1e-5
MODULES, PER, P, PPP = 27, 16, 500, 10
D = MODULES * PER
PARTS = P // PPP
GEOM = dict(n_planes=1, n_fan_det=D, n_fan_proj=P, n_par_proj=128, n_par_det=128, n_pixels=128,
            source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0],
            delta_x=[0.0], delta_z=[1417.0], source_angle=[360.0])


@pytest.fixture(scope="module")
def scan():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return phantom.make_scan(12, 1, P, D, 215.0, 240.0, seed=77, defect_fraction=0.01, distinct=12)


def module_major(frame):
    """[P][D] detector-major -> [modules][P][16] as the detector modules send it."""
    return np.ascontiguousarray(frame.reshape(P, MODULES, PER).transpose(1, 0, 2))


def detector_major(frame_mm):
    return np.ascontiguousarray(frame_mm.reshape(MODULES, P, PER).transpose(1, 0, 2).reshape(P, D))


def packets_of(raw):
    """packets[f][m] = list of (part, bytes) of frame f, module m."""
    out = []
    for f in range(raw.shape[0]):
        mm = module_major(raw[f])
        out.append([[(p, rg.encode_packet(f, p, mm[m, p * PPP:(p + 1) * PPP])) for p in range(PARTS)]
                    for m in range(MODULES)])
    return out


def run_stream(asm, order_of_module):
    """Module threads send their packets (retrying while the ring is full);
    the caller's thread consumes. Returns [(index, module-major frame copy on
    the device)] in hand-out order."""
    errors = []

    def producer(m):
        try:
            for f, part, pkt in order_of_module(m):
                while True:
                    r = asm.ingest(m, pkt)
                    if r != rg.INGEST_RING_FULL:
                        break
                    time.sleep(0.0005)
                if r != rg.INGEST_ACCEPTED:
                    errors.append((m, f, part, r))
        except Exception as e:  # pragma: no cover - reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=producer, args=(m,)) for m in range(MODULES)]
    for t in threads:
        t.start()
    ring_t = asm.ring
    got = []
    done_sending = False
    while True:
        nxt = asm.next(0.2)
        if nxt is None:
            if done_sending:
                break
            if not any(t.is_alive() for t in threads):
                done_sending = True
                asm.finish()
            continue
        idx, slot = nxt
        got.append((idx, ring_t[slot].cuda()))  # one upload from the pinned slot
        torch.cuda.synchronize()
        asm.release(idx)
    for t in threads:
        t.join()
    assert not errors, errors
    return got


def reconstruct_and_check(frames_mm_dev, sc):
    """Engine (module-major input) vs the oracle on the same bytes."""
    n = len(frames_mm_dev)
    g = rg.make_geometry(**GEOM, n_modules=MODULES)
    p = rg.make_params(filter_type="sheppLogan", defects=True, masking=True, module_major=True)
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=n)
    raw = torch.stack(frames_mm_dev).contiguous()
    img = torch.empty((n, GEOM["n_pixels"], GEOM["n_pixels"]), dtype=torch.float32, device="cuda")
    fbp.enqueue(raw, img, 0, n)
    torch.cuda.synchronize()
    got = img.cpu().numpy()
    host = raw.cpu().numpy().view(np.uint16)
    dm = np.stack([detector_major(host[i]) for i in range(n)])
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, 1, 0.67, 1.5, True, oracle.QUIRK_NONE)
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    exp = oracle.fbp(ns(GEOM), op, oracle.f2p_records(ns(GEOM), oracle.QUIRK_NONE), ref, dark, dm,
                     np.zeros(n, np.int32))
    for i in range(n):
        mr, l2 = rel_err(got[i], exp[i])
        assert mr < MAX_REL and l2 < MAX_REL, (i, mr, l2)
    return dm


def test_packets_exact_rule_to_engine(scan):
    raw = scan.raw
    F = raw.shape[0]
    pk = packets_of(raw)
    lost = (5, 3, 7)  # frame, module, part
    layout = rg.packet_layout(MODULES, PER, P, PPP, ring=6)
    ring = torch.zeros((6, MODULES, P, PER), dtype=torch.int16).pin_memory()
    asm = rg.Assembler(layout, ring, skip_lag=2, completion=rg.COMPLETION_EXACT)

    def order(m):
        rng = random.Random(100 + m)
        seq = []
        for f0 in range(0, F, 2):  # two consecutive frames interleaved at random
            win = [(f, part, pkt) for f in (f0, f0 + 1) for part, pkt in pk[f][m] if (f, m, part) != lost]
            rng.shuffle(win)
            seq += win
        return seq

    got = run_stream(asm, order)
    idx = [i for i, _ in got]
    assert idx == [f for f in range(F) if f != lost[0]], idx
    st = asm.stats()
    assert st["skipped"] == 1 and st["duplicates"] == 0, st
    dm = reconstruct_and_check([t for _, t in got], scan)
    np.testing.assert_array_equal(dm, raw[idx])  # every handed-out frame is exactly what was sent


def test_packets_reference_rule_to_engine(scan):
    """Frames are released to the module threads one at a time (each frame's
    packets still arrive concurrently from all modules), so which frame is
    handed out is deterministic; skipping under the newest-common rule is
    covered on the CPU (tests/cpp/test_packets_cpu.cpp)."""
    raw = scan.raw
    F = raw.shape[0]
    pk = packets_of(raw)
    lost = (6, 2, 20)  # a middle part: the module still announces frame 6 with its last part
    layout = rg.packet_layout(MODULES, PER, P, PPP, ring=4)
    ring = torch.zeros((4, MODULES, P, PER), dtype=torch.int16).pin_memory()
    asm = rg.Assembler(layout, ring, completion=rg.COMPLETION_LAST_PART)
    go = [threading.Event() for _ in range(F)]
    errors = []

    def producer(m):
        for f in range(F):
            if not go[f].wait(timeout=60):
                errors.append(("no go", m, f))
                return
            for part, pkt in pk[f][m]:
                if (f, m, part) == lost:
                    continue
                while (r := asm.ingest(m, pkt)) == rg.INGEST_RING_FULL:
                    time.sleep(0.0005)
                if r != (rg.INGEST_STALE if f == 0 else rg.INGEST_ACCEPTED):
                    errors.append((m, f, part, r))

    threads = [threading.Thread(target=producer, args=(m,)) for m in range(MODULES)]
    for t in threads:
        t.start()
    got = []
    try:
        for f in range(F):
            go[f].set()
            nxt = asm.next(0.3 if f == 0 else 20.0)
            if f == 0:
                assert nxt is None, nxt  # the reference's fetch never hands out index 0
                continue
            assert nxt is not None and nxt[0] == f, (f, nxt)
            got.append((f, ring[nxt[1]].cuda()))
            torch.cuda.synchronize()
            asm.release(f)
    finally:
        for e in go:
            e.set()
        for t in threads:
            t.join()
    assert not errors, errors
    asm.finish()
    assert asm.next(0.1) is None
    dm = reconstruct_and_check([t for _, t in got], scan)
    for k, (i, _) in enumerate(got):
        if i == lost[0]:
            # the lost part reads what slot 6 % 4 = 2 held before: frame 2's values
            m, part = lost[1], lost[2]
            rows = slice(part * PPP, (part + 1) * PPP)
            held, sent, before = module_major(dm[k]), module_major(raw[i]), module_major(raw[2])
            np.testing.assert_array_equal(held[m, rows], before[m, rows])
            assert not np.array_equal(held[m, rows], sent[m, rows])
            held[m, rows] = sent[m, rows]
            np.testing.assert_array_equal(held, sent)
        else:
            np.testing.assert_array_equal(dm[k], raw[i])
    assert asm.stats()["skipped"] == 0
