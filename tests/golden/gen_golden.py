"""Generate the golden vectors that pin the CPU oracle to the reference's own kernels.

Runs here, where the reference sources exist: `make -C oracle ref` compiles the reference's
hot-path kernels (MarWo22/master_thesis src/cuda_compute/plate_tectonics_kernel.cu, ccl.cu,
kernel_settings.cu, and the conversion kernels of texture_save.cu) for the CPU, and oracle/ref_harness.cpp launches them with a sequential thread
emulation.  Inputs come from the engine's host-only synthetic generator (deterministic in its
seed).  Outputs are written to tests/golden/*.npz and committed; the tests never need the
reference itself.

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import master_thesis_gb300 as T  # noqa: E402
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def P(a):
    return a.ctypes.data


def ref_settings(kind: str) -> T.Settings:
    """'baseline': the synthetic benchmark parameters; 'reference': the reference's defaults.
    Collision typing thresholds are lowered so that small grids exercise every collision path."""
    s = T.baseline_settings() if kind == "baseline" else T.default_settings()
    s.kernel.minCollisionSize = 3
    s.kernel.collisionTypeUpdateCooldown = 2
    return s


def world(W, H, plates, vel, seed, kind):
    h, ids, pl = T.generate_world(W, H, plates, vel, seed)
    if kind == "reference":  # the reference's height scale: metres around 10000
        h = (np.float32(10000.0) + np.float32(10000.0) * h).astype(np.float32)
    return h, ids, pl


def ref_step_composition(name, W, H, plates, vel, seed, kind, steps, hyd_iters, dt):
    """`steps` steps composed of the reference's kernels in the engine's phase order, uplift
    off and thermal off (the reference's thermal kernel is racy; see the thermal fixture)."""
    R = O.ref()
    st = ref_settings(kind)
    R.ref_set_settings(C.addressof(st.kernel))
    h, ids, pl = world(W, H, plates, vel, seed, kind)
    N = W * H
    w = np.zeros((H, W), np.float32)
    s = np.zeros((H, W), np.float32)
    f = np.zeros((H, W, 4), np.float32)
    bm = np.zeros(T.NUM_PAIRS, np.uint8)
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    wseed = 1000
    rec = {"h0": h.copy(), "id0": ids.copy(), "plates0": pl.copy()}
    for it in range(steps):
        dest = np.zeros(N, np.uint32)
        R.ref_pixel_movements(W, H, P(ids), P(pl), P(dest))
        word = np.zeros(N, np.uint32)
        R.ref_register_collisions(W, H, P(ids), P(dest), P(word))
        R.ref_collision_types(W, H, P(ids), P(h), P(word), P(pl), P(bm))
        hn = np.zeros_like(h)
        idn = np.zeros_like(ids)
        acc = np.zeros_like(ids)
        uh = np.zeros_like(h)
        ut = np.zeros_like(ids)
        R.ref_process_collisions(W, H, P(ids), P(h), P(word), P(pl), P(bm), P(div), wseed, it,
                                 P(hn), P(idn), P(acc), P(uh), P(ut))
        rc = R.ref_hydraulic(W, H, P(hn), P(w), P(s), P(f), hyd_iters, dt, wseed + it)
        assert rc == 0
        R.ref_accretion(W, H, P(hn), P(acc), P(idn))
        # sub-cell centre update of applyPlateMovementChanges (plate_tectonics_kernel.cu:1871-1876)
        cx = pl["pixelCenter_x"] + pl["direction_x"] * pl["velocity"]
        cy = pl["pixelCenter_y"] + pl["direction_y"] * pl["velocity"]
        pl["pixelCenter_x"] = cx - np.floor(cx)
        pl["pixelCenter_y"] = cy - np.floor(cy)
        h, ids = hn, idn
        labels = np.zeros((H, W), np.uint32)
        R.ref_ccl(W, H, P(ids), P(labels))
        for k, v in dict(dest=dest.reshape(H, W), word=word.reshape(H, W), bitmap=bm.copy(), div=div.copy(),
                         h=h.copy(), id=ids.copy(), acc=acc.copy(), w=w.copy(), s=s.copy(), flux=f.copy(),
                         labels=labels, plates=pl.copy()).items():
            rec[f"{k}_{it}"] = v
    np.savez_compressed(OUT / f"{name}.npz", W=W, H=H, steps=steps, hyd_iters=hyd_iters, dt=np.float32(dt),
                        seed=wseed, kind=kind, **rec)
    print("wrote", name, "accretions", sum(int((rec[f'acc_{i}'] > 0).sum()) for i in range(steps)),
          "typed pairs", int((bm != 0).sum()))


def ref_uplift_steps(name, W, H, plates, vel, seed, steps, prop_threshold):
    """The reference uplift (continental propagation, JFA distance field, applyUplift) after each
    of `steps` steps of the reference's collision kernels, in the reference's height units; the
    propagation threshold is lowered so that the continental ray march takes several cells."""
    R = O.ref()
    st = ref_settings("reference")
    st.kernel.continentalPropThreshold = prop_threshold
    R.ref_set_settings(C.addressof(st.kernel))
    h, ids, pl = world(W, H, plates, vel, seed, "reference")
    N = W * H
    bm = np.zeros(T.NUM_PAIRS, np.uint8)
    div = np.zeros(T.NUM_DIV_WORDS, np.uint32)
    wseed = 1000
    rec = {}
    for it in range(steps):
        dest = np.zeros(N, np.uint32)
        R.ref_pixel_movements(W, H, P(ids), P(pl), P(dest))
        word = np.zeros(N, np.uint32)
        R.ref_register_collisions(W, H, P(ids), P(dest), P(word))
        R.ref_collision_types(W, H, P(ids), P(h), P(word), P(pl), P(bm))
        hn = np.zeros_like(h)
        idn = np.zeros_like(ids)
        acc = np.zeros_like(ids)
        uh = np.zeros_like(h)
        ut = np.zeros_like(ids)
        R.ref_process_collisions(W, H, P(ids), P(h), P(word), P(pl), P(bm), P(div), wseed, it,
                                 P(hn), P(idn), P(acc), P(uh), P(ut))
        h_res = hn.copy()
        seeds = np.zeros((H, W), np.int32)
        dists = np.zeros((H, W), np.int32)
        R.ref_uplift(W, H, P(word), P(uh), P(ut), P(h), P(pl), P(idn), P(hn), P(seeds), P(dists))
        for k, v in dict(word=word.reshape(H, W), up_h=uh, up_t=ut, h_old=h.copy(), plates=pl.copy(),
                         id_new=idn.copy(), h_res=h_res, h_up=hn.copy(), seed=seeds, dist=dists,
                         id_old=ids.copy(), bitmap=bm.copy(), div=div.copy()).items():
            rec[f"{k}_{it}"] = v
        R.ref_accretion(W, H, P(hn), P(acc), P(idn))
        cx = pl["pixelCenter_x"] + pl["direction_x"] * pl["velocity"]
        cy = pl["pixelCenter_y"] + pl["direction_y"] * pl["velocity"]
        pl["pixelCenter_x"] = cx - np.floor(cx)
        pl["pixelCenter_y"] = cy - np.floor(cy)
        h, ids = hn, idn
    np.savez_compressed(OUT / f"{name}.npz", W=W, H=H, steps=steps, seed=wseed,
                        prop_threshold=np.float32(prop_threshold), **rec)
    changed = sum(int((rec[f"h_up_{i}"] != rec[f"h_res_{i}"]).sum()) for i in range(steps))
    seeded = sum(int((rec[f"seed_{i}"] >= 0).sum()) for i in range(steps))
    cont = sum(int(((rec[f"up_t_{i}"] & 1) == 1).sum()) for i in range(steps))
    print("wrote", name, "uplifted cells", changed, "cells with a seed", seeded, "continental records", cont)


def ref_thermal_isolated(name, W, H, seed):
    """Thermal on isolated peaks (4 cells apart) with the reference's own parameters (talus
    threshold 0.5 * 1000 m, amplitude 0.5 m): a neighbour receives at most 0.5 m and never becomes
    active, so the reference kernel's in-place updates cannot interfere with each other and its
    result is well defined (and equal to the gather form)."""
    R = O.ref()
    st = T.default_settings()
    R.ref_set_settings(C.addressof(st.kernel))
    rng = np.random.default_rng(seed)
    h = np.full((H, W), np.float32(8000.0), np.float32)
    for y in range(1, H, 4):
        for x in range(1, W, 4):
            if rng.random() < 0.7:
                h[y, x] = np.float32(8000.0 + rng.uniform(300.0, 3000.0))
            for dy in (-1, 0, 1):  # foothills: some directions of a peak fall below the talus
                for dx in (-1, 0, 1):  # threshold; a foothill is never itself 500 m above flat land
                    if (dy or dx) and rng.random() < 0.3:
                        h[(y + dy) % H, (x + dx) % W] = np.float32(8000.0 + rng.uniform(0.0, 400.0))
    out = h.copy()
    R.ref_thermal(W, H, P(out))
    np.savez_compressed(OUT / f"{name}.npz", W=W, H=H, h_in=h, h_out=out)
    print("wrote", name, "changed cells", int((out != h).sum()))


def ref_ccl_cases(name):
    """Reference CCL labels on structured id maps that exercise wrap and diagonal links."""
    R = O.ref()
    cases = {}
    rng = np.random.default_rng(5)
    H, W = 32, 48
    cases["random4"] = rng.integers(0, 4, (H, W)).astype(np.uint8)
    cases["random2"] = rng.integers(0, 2, (H, W)).astype(np.uint8)
    d = np.zeros((H, W), np.uint8)
    for k in range(-H, W):
        for y in range(H):
            x = y + k
            if 0 <= x < W and (k % 5 == 0):
                d[y, x] = 1
    cases["diagonals"] = d
    a = np.zeros((H, W), np.uint8)
    a[::3, :] = 1
    a[:, ::7] = 2
    cases["stripes"] = a
    _, ids, _ = T.generate_world(W, H, 6, 1.0, 11)
    cases["voronoi"] = ids
    out = {}
    for k, ids in cases.items():
        lab = np.zeros((H, W), np.uint32)
        R.ref_ccl(W, H, P(ids), P(lab))
        out[f"{k}_id"] = ids
        out[f"{k}_labels"] = lab
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print("wrote", name)


def ref_export(name):
    """The reference's image conversions (texture_save.cu): the colour of every plate id (a 16 x 16
    map of ids 0..255) and the 16-bit grey of heights around, at and beyond the default
    minUpliftClamp / maxUpliftClamp range and of random heights over another range."""
    R = O.ref()
    ids = np.arange(256, dtype=np.uint8).reshape(16, 16)
    rgb = np.zeros((16, 16, 3), np.uint8)
    R.ref_ids_rgb(16, 16, P(ids), P(rgb))
    st = T.default_settings()
    lo, hi = float(st.kernel.minUpliftClamp), float(st.kernel.maxUpliftClamp)
    span = hi - lo
    edge = np.array([lo - 1.0, lo, np.nextafter(np.float32(lo), np.float32(hi)), lo + span * 0.25, lo + span * 0.5,
                     np.nextafter(np.float32(hi), np.float32(lo)), hi, hi + 1.0, -3.0e38, 3.0e38, 0.0, -0.0],
                    np.float32)
    rng = np.random.default_rng(17)
    h1 = np.concatenate([edge, rng.uniform(lo - 0.1 * span, hi + 0.1 * span, 1024 - edge.size).astype(np.float32)])
    h1 = h1.reshape(32, 32)
    g1 = np.zeros((32, 32), np.uint16)
    R.ref_gray16(32, 32, P(h1), lo, hi, P(g1))
    h2 = rng.normal(0.0, 400.0, (24, 40)).astype(np.float32)
    g2 = np.zeros((24, 40), np.uint16)
    R.ref_gray16(40, 24, P(h2), -1000.0, 1000.0, P(g2))
    np.savez_compressed(OUT / f"{name}.npz", ids=ids, rgb=rgb, h1=h1, lo1=np.float32(lo), hi1=np.float32(hi), g1=g1,
                        h2=h2, lo2=np.float32(-1000.0), hi2=np.float32(1000.0), g2=g2)
    print("wrote", name)


def ref_dynamics(name):
    """Plate dynamics kernels of the reference: processCollisions' friction per plate on an evolved
    world, the angular geometric centres, computeCurl of a pressure texture and
    applyPlateMovementChanges on given plate records."""
    R = O.ref()
    W, H = 64, 64
    st = T.baseline_settings()
    st.kernel.minCollisionSize = 3
    st.kernel.collisionTypeUpdateCooldown = 2
    st.kernel.frictionCoefficientContinental = 0.3
    st.kernel.frictionCoefficientSubduction = 0.05
    st.kernel.frictionCoefficientAccretion = 0.15
    R.ref_set_settings(C.addressof(st.kernel))
    h, ids, pl = T.generate_world(W, H, 7, 1.5, 23)
    ow = O.OracleWorld(st, h, ids, pl, 1000)
    ow.step(3)
    # the collide phases of the next step, from the oracle (pinned by the step compositions)
    offx, offy, _ = O.plate_offsets(ow.plates)
    _, word, _, _ = O.collision_words(ow.id, offx, offy)
    bitmap = O.collision_types(word, ow.h, offx, offy, st, ow.bitmap)
    dyn = O.plate_stats(ow.h, ow.id, 3)
    mass = np.ascontiguousarray(dyn["mass"], np.float32)
    fric = np.zeros(255, np.float32)
    R.ref_collision_friction(W, H, P(ow.id), P(ow.h), P(word), P(ow.plates), P(mass), P(bitmap), P(ow.div), 1000, 3,
                             P(fric))
    # centres: the evolved ids, and a map with plates across both seams
    centres = np.zeros((255, 2), np.float32)
    R.ref_plate_centres(W, H, P(ow.id), P(centres))
    ids2 = np.full((50, 70), 3, np.uint8)  # plates 1 and 2 straddle the seams; 3 is the background
    ids2[:30, :12] = 1
    ids2[:30, 61:] = 1
    ids2[:8, 20:40] = 2
    ids2[44:, 20:40] = 2
    centres2 = np.zeros((255, 2), np.float32)
    R.ref_plate_centres(70, 50, P(ids2), P(centres2))
    # curl of a random pressure texture, nearest-scaled from 40 x 28 to 64 x 64
    rng = np.random.default_rng(29)
    pressure = rng.random((28, 40)).astype(np.float32)
    curl = np.zeros((H, W, 2), np.float32)
    R.ref_curl(40, 28, P(pressure), W, H, P(curl))
    # movement changes on synthetic records
    plates_in = ow.plates.copy()
    dyn_in = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    dyn_in["velocitySmoothed"] = rng.uniform(0.0, 1.0, 255)
    ang = rng.uniform(0.0, 2 * np.pi, 255)
    dyn_in["directionSmoothed_x"] = np.cos(ang)
    dyn_in["directionSmoothed_y"] = np.sin(ang)
    dyn_in["geometricCenter_x"] = rng.uniform(0.0, W, 255)
    dyn_in["geometricCenter_y"] = rng.uniform(0.0, H, 255)
    dyn_in["mergeWaitTime"] = rng.integers(0, 3, 255)
    fric_in = rng.uniform(0.0, 0.5, 255).astype(np.float32)
    fric_in[:20] = 0.0
    plates_out, dyn_out = plates_in.copy(), dyn_in.copy()
    R.ref_plate_motion(W, H, P(plates_out), P(dyn_out), P(fric_in), P(curl))
    np.savez_compressed(OUT / f"{name}.npz", W=W, H=H, ids=ow.id, h=ow.h, word=word, plates=ow.plates,
                        bitmap=bitmap, div=ow.div, mass=mass, friction=fric, centres=centres, ids2=ids2,
                        centres2=centres2, pressure=pressure, curl=curl, plates_in=plates_in, dyn_in=dyn_in,
                        fric_in=fric_in, plates_out=plates_out, dyn_out=dyn_out,
                        fc=np.float32([0.3, 0.05, 0.15]))
    print("wrote", name, "plates with friction", int((fric != 0).sum()))


def ref_init(name):
    """The reference's initPlateIDs and initHeightmap for seeds of the reference's draws (two
    Voronoi generations, a non-square world, so the swapped position ranges show)."""
    R = O.ref()
    out = {}
    for tag, (W, H, seed, plates, gens) in {"a": (96, 64, 1234, 12, (60, 150)), "b": (50, 80, 7, 5, ())}.items():
        sx, sy, sid, pl, dy = O.reference_seeds(W, H, seed, plates, gens)
        h = np.zeros((H, W), np.float32)
        ids = np.zeros((H, W), np.uint8)
        R.ref_init(W, H, seed, P(sx), P(sy), P(sid), len(sx), P(h), P(ids))
        out.update({f"{tag}_W": W, f"{tag}_H": H, f"{tag}_seed": seed, f"{tag}_plates": plates,
                    f"{tag}_gens": np.array(gens, np.int32), f"{tag}_sx": sx, f"{tag}_sy": sy, f"{tag}_sid": sid,
                    f"{tag}_h": h, f"{tag}_ids": ids})
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print("wrote", name)


def ref_policy(name):
    """mergePlates with the reference's kernels (getNeighboringPlates, getPlateMerges in thread order,
    clearCollisionTypes per parent, the remap of mergeAndCountSizeMass) on a ten-plate map whose
    records make some pairs merge, some compete for the same plate, one wait and one exceed the
    area cap."""
    R = O.ref()
    st = T.baseline_settings()
    st.kernel.mergeMinVelocity = 0.2
    st.kernel.mergeDotDirectionThreshold = 0.9
    st.kernel.mergeVelocityDiffThreshold = 0.1
    st.kernel.targetMaximumPlateArea = 900
    R.ref_set_settings(C.addressof(st.kernel))
    W, H = 60, 40
    _, ids, _ = T.generate_world(W, H, 10, 1.0, 31)
    rng = np.random.default_rng(37)
    pl = np.zeros(255, T.PLATE_DTYPE)
    dy = np.zeros(255, T.PLATE_DYNAMICS_DTYPE)
    ang = rng.uniform(0, 2 * np.pi, 10)
    ang[[1, 2, 3]] = ang[0] + rng.uniform(-0.2, 0.2, 3)  # aligned with plate 0
    for k in range(10):
        pl[k]["velocity"] = rng.uniform(0.05, 0.6)
        pl[k]["direction_x"], pl[k]["direction_y"] = np.cos(ang[k]), np.sin(ang[k])
        dy[k]["velocitySmoothed"] = pl[k]["velocity"] + rng.uniform(-0.05, 0.05)
        dy[k]["directionSmoothed_x"], dy[k]["directionSmoothed_y"] = np.cos(ang[k]), np.sin(ang[k])
        dy[k]["size"] = int((ids == k).sum())
        dy[k]["mass"] = float(rng.uniform(100, 1000))
    dy[7]["mergeWaitTime"] = 2
    pl[[5, 6]]["velocity"] = 0.1  # slow pair candidates
    bitmap = rng.integers(0, 256, 32385).astype(np.uint8)
    out_ids, out_bm = ids.copy(), bitmap.copy()
    merge_ids = np.zeros(255, np.int32)
    R.ref_merges(W, H, P(out_ids), P(pl), P(dy), P(out_bm), P(merge_ids))
    np.savez_compressed(OUT / f"{name}.npz", ids=ids, plates=pl, dyn=dy, bitmap=bitmap, out_ids=out_ids,
                        out_bitmap=out_bm, merge_ids=merge_ids,
                        ks=np.float32([0.2, 0.9, 0.1, 900]))
    print("wrote", name, "merges", int((merge_ids == -1).sum()))


def main():
    O.build(ref=True)
    ref_step_composition("ref_steps_baseline_64x64", 64, 64, 8, 1.0, 7, "baseline", 6, 20, 0.02)
    ref_step_composition("ref_steps_baseline_128x48", 128, 48, 5, 1.0, 3, "baseline", 6, 20, 0.02)
    ref_step_composition("ref_steps_reference_64x64", 64, 64, 8, 1.0, 9, "reference", 6, 10, 1.0)
    ref_uplift_steps("ref_uplift_64x48", 64, 48, 8, 1.5, 21, 5, 12000.0)
    ref_thermal_isolated("ref_thermal_isolated_64x64", 64, 64, 13)
    ref_ccl_cases("ref_ccl_cases")
    ref_export("ref_export")
    ref_dynamics("ref_dynamics")
    ref_init("ref_init")
    ref_policy("ref_policy")


if __name__ == "__main__":
    main()
