"""CPU restatement of the lane-slice arithmetic of the warp's segment tests
(refine_pixel_pair, farm_gb300/csrc/segments.cuh).

A group of R source segments (R < 32 for a pixel's last group or a small
pixel) is repeated over G = floor(32 / R) slices of lanes; in each staged
chunk of m target vertices, slice g walks vertices [j0, j1) with
q = ceil(m / G), j0 = min(m, g q), j1 = min(m, j0 + q), starting from the
vertex before j0. The target segment ending at vertex j is tested by the
lanes whose slice holds j, against the segment from vertex j - 1 (the
previous chunk's last vertex for j = 0). This checks, for every R and m,
that each (source segment, target vertex) pair is visited exactly once, and
that the per-lane test count the kernel adds up (the predecessor's segment
bit over [j0 - 1, j1 - 2], plus the carried bit for j0 = 0) counts exactly
the visited vertices whose predecessor starts a segment."""
import random


def popc(x):
    return bin(x & 0xFFFFFFFF).count("1")


def test_slices_cover_each_pair_once_and_count_tests():
    rng = random.Random(5)
    for R in range(1, 33):
        G = 32 // R
        for m in range(1, 33):
            segmask = rng.getrandbits(32) & ((1 << m) - 1)
            pseg0 = rng.random() < 0.5
            seen = {}
            counted = 0
            expected = 0
            for lane in range(32):
                slc, seg = lane // R, lane % R
                valid = slc < G
                q = (m + G - 1) // G
                j0 = min(m, slc * q) if valid else m
                j1 = min(m, j0 + q)
                for j in range(j0, j1):
                    seen[(seg, j)] = seen.get((seg, j), 0) + 1
                    pred = pseg0 if j == 0 else bool((segmask >> (j - 1)) & 1)
                    expected += int(pred)
                if valid and j1 > j0:
                    below = 0xFFFFFFFF if j1 - 1 > 31 else (1 << (j1 - 1)) - 1
                    frm = ~((1 << (j0 - 1)) - 1) & 0xFFFFFFFF if j0 > 0 else 0xFFFFFFFF
                    counted += (1 if (j0 == 0 and pseg0) else 0) + popc(segmask & below & frm)
            assert all(seen.get((s, j), 0) == 1 for s in range(R) for j in range(m)), (R, m)
            assert len(seen) == R * m
            assert counted == expected, (R, m)
