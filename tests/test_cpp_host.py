"""The C++ host layer (the reference's class interface over the C ABI).

CPU: the reference's own applications compile and link unchanged against it (when the reference
sources are present); estimator applications replay the CPU oracle's traces bit for bit through
ZGraphInstance::replay_trace; without a GPU a program fails loudly instead of falling back.
GPU: tests/cpp/zgh_gpu_check.cpp runs the applications end to end (identification, calculate,
ErrorProfile, TimeProfile, AllPredicate, the 3-motif cache, SamplerGenerator) and compares every
result with the C ABI run on the same draws."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import zgbuild
import zgraph as Z

HERE = os.path.dirname(os.path.abspath(__file__))
CPP = os.path.join(HERE, "cpp")
# the reference's sources (present where the oracle's reference drivers are built; absent on the GPU host)
REF_APPS = os.path.join(os.environ.get("ZG_REFERENCE_DIR", "/root/reference"), "applications")


def _build(src, out):
    return zgbuild.build_app([os.path.join(CPP, src)], out, include_dirs=[CPP])


@pytest.mark.skipif(not os.path.isdir(REF_APPS), reason="reference sources not present")
def test_reference_applications_compile_unchanged(tmp_path):
    apps = sorted(f for f in os.listdir(REF_APPS) if f.endswith(".cpp"))
    assert len(apps) >= 13
    for a in apps:
        zgbuild.build_app([os.path.join(REF_APPS, a)], str(tmp_path / a[:-4]))
        assert os.path.exists(tmp_path / a[:-4])


HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])


def _write_graph(d, edges, nv):
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "graph.bin"), "wb") as f:
        f.write(np.uint64(len(edges)).tobytes())
        f.write(np.uint32(nv).tobytes())
        f.write(np.ascontiguousarray(edges, np.uint32).tobytes())


def _keep_hits(og, prog, seed, stream, chunks):
    """The first 4096 samples as they come, then hits only (rare patterns need many samples)."""
    parts, hits = [], 0
    for k in range(chunks):
        tr, _ = O.traces(og, prog, 1 << 17, seed, stream=stream, first=k << 17)
        if k == 0:
            parts.append(tr[:4096])
            tr = tr[4096:]
        h = tr[tr["hit"] != 0][:4096 - hits]
        parts.append(h)
        hits += len(h)
        if hits >= 4096:
            break
    return np.concatenate(parts)


def _write_case(d, edges, nv):
    _write_graph(d, edges, nv)
    og = O.OracleGraph(edges, nv)
    progs = {
        "triangle": O.OracleProgram(1), "four_clique": O.OracleProgram(2), "three_chain": O.OracleProgram(3),
        "four_chain": O.OracleProgram(4), "chain5": O.OracleProgram(5, 5), "chain3": O.OracleProgram(5, 3),
        "pattern_star": O.OracleProgram(6, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)])),
        "pattern_triangle": O.OracleProgram(6, pattern=(3, [(0, 1), (0, 2), (1, 2)])),
    }
    for i, (name, p) in enumerate(progs.items()):
        _keep_hits(og, p, 91 + i, i, 1).tofile(os.path.join(d, name + ".tr"))
    # the house needs a dense graph: about one hit in 10^4 samples on G(10, 0.6)
    rng = np.random.default_rng(3)
    iu = np.triu_indices(10, 1)
    mask = rng.random(len(iu[0])) < 0.6
    dense = np.stack([iu[0][mask], iu[1][mask]], 1).astype(np.uint32)
    rng.shuffle(dense)
    _write_graph(os.path.join(d, "house"), dense, 10)
    tr = _keep_hits(O.OracleGraph(dense, 10), O.OracleProgram(6, pattern=HOUSE), 7, 3, 8)
    tr.tofile(os.path.join(d, "house", "pattern_house.tr"))


def test_applications_replay_oracle_traces(tmp_path):
    exe = _build("zgh_replay_check.cpp", str(tmp_path / "zgh_replay_check"))
    e = Z.gen_rmat(9, 12, seed=17)
    _write_case(str(tmp_path), e, 1 << 9)
    p = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    print(p.stdout)
    assert p.returncode == 0 and "PASS" in p.stdout, p.stdout


def test_without_gpu_fails_loudly(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = _build("zgh_gpu_check.cpp", str(tmp_path / "zgh_gpu_check"))
    p = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert p.returncode != 0
    assert "zg_init" in p.stdout, p.stdout


@pytest.mark.gpu
def test_applications_end_to_end_on_gpu(tmp_path):
    exe = _build("zgh_gpu_check.cpp", str(tmp_path / "zgh_gpu_check"))
    p = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=1200)
    print(p.stdout)
    assert p.returncode == 0 and "PASS" in p.stdout, p.stdout
