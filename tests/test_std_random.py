"""The oracle's restatement of libstdc++'s default_random_engine + normal_distribution<float>
(the reference's host far-failure draws, src/coredynamics.cu:195, 319) against libstdc++
itself, compiled here with g++: one shared distribution, draws alternating between engines so
that cached second values cross engines as they do in recal_G_vec."""
import ctypes as C
import shutil
import subprocess

import numpy as np
import pytest

CPP = r"""
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
int main() {
    int nEng, n;
    if (scanf("%d %d", &nEng, &n) != 2) return 1;
    std::vector<std::default_random_engine> e(nEng);
    for (int q = 0; q < nEng; q++) { unsigned long long s; if (scanf("%llu", &s) != 1) return 1; e[q].seed(s); }
    std::normal_distribution<float> d(0.0, 1.0);
    for (int q = 0; q < n; q++) {
        int w; if (scanf("%d", &w) != 1) return 1;
        float v = d(e[w]); unsigned u; std::memcpy(&u, &v, 4); printf("%08x\n", u);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def stdlib_draws(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("stdrand")
    src, exe = d / "draws.cpp", d / "draws"
    src.write_text(CPP)
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe), str(src)], check=True)

    def run(seeds, who):
        inp = f"{len(seeds)} {len(who)}\n" + " ".join(str(int(s)) for s in seeds) + "\n" + \
              " ".join(str(int(w)) for w in who) + "\n"
        out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split()
        return np.array([int(x, 16) for x in out], dtype=np.uint32).view(np.float32)
    return run


def oracle_draws(seeds, who):
    import oracle
    s = np.ascontiguousarray(seeds, dtype=np.uint64)
    w = np.ascontiguousarray(who, dtype=np.int32)
    out = np.empty(len(w), np.float32)
    oracle.lib().orc_std_normal_draws(s.ctypes.data_as(C.POINTER(C.c_uint64)), len(s),
                                      w.ctypes.data_as(C.POINTER(C.c_int32)), len(w),
                                      out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def test_std_normal_matches_libstdcxx(stdlib_draws):
    rng = np.random.default_rng(3)
    seeds = [0, 1, 2147483647, 2147483648, 12345, 2**40 + 7, 987654321]
    who = rng.integers(0, len(seeds), 4000)
    ref = stdlib_draws(seeds, who)
    np.testing.assert_array_equal(oracle_draws(seeds, who), ref)


def test_std_normal_one_engine_sequence(stdlib_draws):
    seeds = [42]
    who = np.zeros(3001, np.int64)
    np.testing.assert_array_equal(oracle_draws(seeds, who), stdlib_draws(seeds, who))


SAMPLE_CPP = r"""
#include <algorithm>
#include <cstdio>
#include <iterator>
#include <random>
#include <vector>
int main() {
    unsigned long long seed; unsigned nblock, bs, nE, k;
    if (scanf("%llu %u %u %u %u", &seed, &nblock, &bs, &nE, &k) != 5) return 1;
    std::vector<unsigned> exc, ids;
    for (unsigned i = 0; i < nblock; i++) for (unsigned j = 0; j < nE; j++) exc.push_back(i * bs + j);
    std::default_random_engine g(seed);
    std::sample(exc.begin(), exc.end(), std::back_inserter(ids), k, g);
    for (unsigned v : ids) printf("%u\n", v);
    return 0;
}
"""


def test_sample_ids_match_std_sample(tmp_path):
    """pv1_sample_ids (minimal output's sampled neurons) equals std::sample over the
    excitatory ids with a default_random_engine, as the reference draws them."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from visual_cortex_gb300 import _native as N
    src, exe = tmp_path / "s.cpp", tmp_path / "s"
    src.write_text(SAMPLE_CPP)
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe), str(src)], check=True)
    for seed, nblock, bs, nE, k in ((7, 2, 8, 6, 5), (123456789, 32, 1024, 768, 4000), (3, 4, 64, 48, 100)):
        ref = subprocess.run([str(exe)], input=f"{seed} {nblock} {bs} {nE} {k}", capture_output=True, text=True,
                             check=True).stdout.split()
        out = np.zeros(nblock * nE, np.uint32)
        n = C.c_uint32()
        assert N.lib.pv1_sample_ids(seed, nblock, bs, nE, k, N.uptr(out), C.byref(n)) == 0
        np.testing.assert_array_equal(out[:n.value], np.array(ref, np.uint32))
