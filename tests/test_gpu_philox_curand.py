"""Philox4x32-10 against NVIDIA's own: cuRAND's device API
(curandStatePhilox4_32_10_t, curand_init + curand4) on the GPU must give
the same four words as the oracle's Philox (which the library's device code
is checked against bit for bit elsewhere) for the counters the jitter uses.

cuRAND's state: key = (seed low, seed high); skipahead_sequence(n) adds n to
the counter's high 64 bits, skipahead(4*m) adds m to its low 64 bits.  The
jitter counter (agent id, step low, step high, stream) is therefore reached
with subsequence = stream << 32 | step_high and a low counter of
step_low << 32 | id.  The test program is compiled here with nvcc for
sm_103a."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SRC = r"""
#include <cstdio>
#include <curand_kernel.h>

// low: the counter's low 64 bits; skipahead takes 4 x counters in 64 bits,
// so they are added in chunks of at most 2^61
__global__ void draw(const unsigned long long* seed, const unsigned long long* subseq,
                     const unsigned long long* low, uint4* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed[i], subseq[i], 0ull, &st);
    unsigned long long left = low[i];
    while (left > 0ull) {
        const unsigned long long c = left < (1ull << 61) ? left : (1ull << 61);
        skipahead(4ull * c, &st);
        left -= c;
    }
    out[i] = curand4(&st);
}

int main() {
    int n = 0;
    if (scanf("%d", &n) != 1 || n <= 0 || n > 4096) return 2;
    unsigned long long hs[4096], hq[4096], ho[4096];
    for (int i = 0; i < n; ++i)
        if (scanf("%llu %llu %llu", &hs[i], &hq[i], &ho[i]) != 3) return 2;
    unsigned long long *ds, *dq, *dof;
    uint4* dout;
    cudaMalloc(&ds, n * 8); cudaMalloc(&dq, n * 8); cudaMalloc(&dof, n * 8);
    cudaMalloc(&dout, n * 16);
    cudaMemcpy(ds, hs, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dq, hq, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dof, ho, n * 8, cudaMemcpyHostToDevice);
    draw<<<(n + 127) / 128, 128>>>(ds, dq, dof, dout, n);
    uint4 out[4096];
    if (cudaMemcpy(out, dout, n * 16, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    for (int i = 0; i < n; ++i) printf("%u %u %u %u\n", out[i].x, out[i].y, out[i].z, out[i].w);
    return 0;
}
"""


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not found")


def test_philox_matches_curand(gpu, tmp_path):
    src = tmp_path / "curand_philox.cu"
    exe = tmp_path / "curand_philox"
    src.write_text(SRC)
    subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", str(src), "-o",
                    str(exe)], check=True, capture_output=True, timeout=300)
    rng = np.random.default_rng(12)
    cases = []
    for k in range(512):
        seed = int(rng.integers(0, 2**64, dtype=np.uint64))
        ident = int(rng.integers(0, 2**32, dtype=np.uint64))
        step = int(rng.integers(0, 2**40, dtype=np.uint64)) if k % 2 else int(rng.integers(0, 5000))
        stream = k % 2
        cases.append((seed, ident, step, stream))
    cases += [(0, 0, 0, 0), (2**64 - 1, 2**32 - 1, 2**64 - 1, 1), (42, 7, 0, 0)]
    lines = [str(len(cases))]
    for seed, ident, step, stream in cases:
        subseq = (stream << 32) | (step >> 32)
        low = ((step & 0xFFFFFFFF) << 32) | ident
        lines.append(f"{seed} {subseq} {low}")
    r = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    got = np.array([[int(v) for v in ln.split()] for ln in r.stdout.strip().splitlines()],
                   dtype=np.uint64)
    assert got.shape == (len(cases), 4)
    for (seed, ident, step, stream), row in zip(cases, got):
        ctr = [ident, step & 0xFFFFFFFF, step >> 32, stream]
        key = [seed & 0xFFFFFFFF, seed >> 32]
        want = oracle.philox(ctr, key)
        assert [int(v) for v in want] == [int(v) for v in row], (seed, ident, step, stream)
