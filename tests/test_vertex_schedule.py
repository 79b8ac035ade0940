"""The vertex phase's per-lane schedule (vertex_warp_schedule in
csrc/acg_vschedule.h), compiled on the host and checked on random patterns:
every (staged vertex, pattern vertex) MU_raw sum is one job on one lane, its
terms in the tile form's order (-CV, then F over the in-edges ascending, then R
over the out-edges ascending), with the right first/last flags and slot on every
word; padding comes only after a lane's last job; the lanes hold a multiple of
four terms and are balanced to within one job of the average."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "application_classification_gb300" / "csrc"

PROBE = r"""
#include <cstdio>
#include <vector>
#include "acg_vschedule.h"
// stdin: cases, then per case "vps pn pe pp pnp" and pe lines "src dst";
// stdout per case: the terms per lane, then the words
int main() {
  int cases;
  if (std::scanf("%d", &cases) != 1) return 1;
  for (int c = 0; c < cases; ++c) {
    int vps, pn, pe, pp, pnp;
    if (std::scanf("%d %d %d %d %d", &vps, &pn, &pe, &pp, &pnp) != 5) return 1;
    std::vector<int> pat(2 * pe + 2 * (pn + 1) + 2 * pe, 0);
    int* ps = pat.data();
    int* pd = ps + pe;
    int* inoff = pd + pe;
    int* inq = inoff + pn + 1;
    int* outoff = inq + pe;
    int* outq = outoff + pn + 1;
    for (int q = 0; q < pe; ++q) {
      if (std::scanf("%d %d", &ps[q], &pd[q]) != 2) return 1;
      inoff[pd[q] + 1]++;
      outoff[ps[q] + 1]++;
    }
    for (int p = 0; p < pn; ++p) {
      inoff[p + 1] += inoff[p];
      outoff[p + 1] += outoff[p];
    }
    std::vector<int> ci(inoff, inoff + pn), co(outoff, outoff + pn);
    for (int q = 0; q < pe; ++q) {
      inq[ci[pd[q]]++] = q;
      outq[co[ps[q]]++] = q;
    }
    std::vector<uint32_t> w;
    const int nt = acg::vertex_warp_schedule(pat.data(), pn, pe, pp, pnp, vps, &w);
    std::printf("%d %zu\n", nt, w.size());
    for (uint32_t x : w) std::printf("%u\n", x);
  }
  std::printf("flags %u %u\n", acg::kSchedStart, acg::kSchedEnd);
  return 0;
}
"""


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("vsched")
    src = d / "probe.cpp"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    return exe


def _run(exe, cases):
    lines = [str(len(cases))]
    for vps, pn, pp, pnp, edges in cases:
        lines.append(f"{vps} {pn} {len(edges)} {pp} {pnp}")
        lines += [f"{s} {d}" for s, d in edges]
    out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", check=True,
                         capture_output=True, text=True).stdout.split()
    res, i = [], 0
    for _ in cases:
        nt, n = int(out[i]), int(out[i + 1])
        res.append((nt, np.array(out[i + 2:i + 2 + n], dtype=np.uint64).astype(np.uint32)))
        i += 2 + n
    assert out[i] == "flags"
    return res, int(out[i + 1]), int(out[i + 2])


def _pads(pn, pe, width):
    """The plan's padded row lengths: edge columns to a multiple of 16 bytes
    (at least one 16-byte unit), pattern-vertex columns likewise."""
    pp = max(width, -(-pe // width) * width)
    pnp = -(-pn // width) * width
    return pp, pnp


def _random_cases(seed):
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(60):
        pn = int(rng.integers(1, 65)) if k % 3 else int(rng.integers(1, 33))
        pe = int(rng.integers(0, 65))
        width = 4 if k % 2 == 0 else 2  # FP32 / FP64 rows
        pp, pnp = _pads(pn, pe, width)
        if pp > 64:
            pe = 64 - (64 % width)
            pp, pnp = _pads(pn, pe, width)
        if k % 5 == 0:  # a hub: many edges into / out of one vertex
            hub = int(rng.integers(0, pn))
            edges = [(hub, int(rng.integers(0, pn))) if rng.random() < 0.5 else (int(rng.integers(0, pn)), hub)
                     for _ in range(pe)]
        else:
            edges = [(int(rng.integers(0, pn)), int(rng.integers(0, pn))) for _ in range(pe)]
        vps = int(rng.choice([1, 2, 4]))
        cases.append((vps, pn, pp, pnp, edges))
    # fixed shapes: the planted 32/64 pattern's size, a path, a star, isolated vertices
    cases.append((4, 32, 64, 32, [(i, (i * 7 + 3) % 32) for i in range(32)] + [(i, (i + 1) % 32) for i in range(32)]))
    cases.append((4, 16, 16, 16, [(i, i + 1) for i in range(15)]))
    cases.append((4, 64, 64, 64, [(0, i) for i in range(1, 64)]))
    cases.append((4, 5, 4, 8, []))
    cases.append((4, 1, 4, 4, [(0, 0), (0, 0)]))
    return cases


def test_schedule_invariants(probe):
    cases = _random_cases(7)
    res, START, END = _run(probe, cases)
    for (vps, pn, pp, pnp, edges), (nt, words) in zip(cases, res):
        assert nt > 0 and nt % 4 == 0 and words.size == nt * 32
        ppl = 1 if pn <= 32 else 2
        oM, oY, oC = 0, vps * pp, 4 * vps * pp  # the stage's M, Y and CV rows
        ins = [[q for q, (s, d) in enumerate(edges) if d == p] for p in range(pn)]
        outs = [[q for q, (s, d) in enumerate(edges) if s == p] for p in range(pn)]
        seen = set()
        loads = []
        lanes = words.reshape(nt // 4, 32, 4).transpose(1, 0, 2).reshape(32, nt)
        for lane in lanes:
            t = 0
            load = 0
            while t < nt and lane[t] & START:
                w0 = int(lane[t])
                slot = w0 >> 16
                jv, p = divmod(slot, 32 * ppl + 1)
                assert 0 <= jv < vps and 0 <= p < pn
                assert (jv, p) not in seen
                seen.add((jv, p))
                want = ([oC + jv * pnp + p] + [oM + jv * pp + q for q in ins[p]]
                        + [oY + jv * pp + q for q in outs[p]])
                got = lane[t:t + len(want)]
                assert got.size == len(want)
                assert [int(x) & 0xFFF for x in got] == want
                assert all(int(x) >> 16 == slot for x in got)
                flags = [int(x) & (START | END) for x in got]
                if len(want) == 1:
                    assert flags == [START | END]
                else:
                    assert flags == [START] + [0] * (len(want) - 2) + [END]
                t += len(want)
                load += len(want)
            # after the lane's last job: padding words only
            assert np.all(lane[t:] == 0)
            loads.append(load)
        assert seen == {(jv, p) for jv in range(vps) for p in range(pn)}
        total = sum(loads)
        assert total == vps * (pn + 2 * len(edges))
        longest = max(1 + len(ins[p]) + len(outs[p]) for p in range(pn))
        # longest first, each to the least loaded lane: no lane ends a job
        # more than one job past the average
        assert max(loads) <= total / 32 + longest
        assert nt == -(-max(loads) // 4) * 4


def test_schedule_tile_form_shapes(probe):
    """More than 64 pattern vertices or padded edge columns take the tile form,
    and so does a stage whose slots (9 bits) or offsets (12 bits) would not fit
    the schedule word."""
    cases = [(4, 65, 4, 68, [(0, 1)]), (4, 10, 68, 12, [(0, 1)] * 65),
             (8, 40, 64, 40, [(0, 1)] * 60),   # slots 8 x 65 > 512
             (15, 32, 64, 32, [(0, 1)] * 60)]  # CV offsets 15 x (4 x 64 + 32) > 4096
    res, _, _ = _run(probe, cases)
    for nt, words in res:
        assert nt == 0 and words.size == 0
