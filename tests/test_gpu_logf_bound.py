"""The FP32 js screen takes its logarithms from the __logf intrinsic and its
error bound from twice the intrinsic's documented accuracy: at most
2^-20.41 absolute error for x in [0.5, 2], at most 6 ulp elsewhere (a sampled
check of the documented figures themselves found a few inputs 6 % beyond
them).  This test checks that allowance on the GPU for every FP32 input the
screen can see (S = P + Q with P, Q in [2^-100, 2^100]): all 2^23
significands of every binade of [2^-100, 2^102), each compared with the FP64
logarithm.  A probe is compiled with the library's own nvcc flags (sm_103a,
-O3, no fast-math) and run once."""
import os
import shutil
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

PROBE = r"""
#include <cstdio>
#include <cmath>
__global__ void k_sweep(int e0, int nbin, int per, unsigned long long* bad, unsigned long long* worst_bits) {
  const long long total = (long long)nbin * per;
  double wmax = 0.0;
  unsigned long long nbad = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int e = e0 + (int)(t / per);
    const int m = (int)(t % per);
    const float x = ldexpf(1.0f + (float)m / (float)per, e);
    const float L = __logf(x);
    const double ex = log((double)x);
    double lim;
    if (x >= 0.5f && x <= 2.0f) {
      lim = ldexp(1.0, -20) * exp2(-0.41);
    } else {
      const float y = fabsf((float)ex);
      lim = 6.0 * ((double)nextafterf(y, INFINITY) - (double)y);
    }
    const double r = fabs((double)L - ex) / lim;
    if (!(r <= 1.0)) ++nbad;
    wmax = fmax(wmax, r);
  }
  if (nbad) atomicAdd(bad, nbad);
  atomicMax(worst_bits, (unsigned long long)__double_as_longlong(wmax));   // >= 0: bits order as values
}
int main() {
  unsigned long long *bad, *worst;
  cudaMalloc(&bad, 8); cudaMalloc(&worst, 8);
  cudaMemset(bad, 0, 8); cudaMemset(worst, 0, 8);
  k_sweep<<<152 * 32, 256>>>(-100, 202, 1 << 23, bad, worst);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long hb = 0, hw = 0;
  cudaMemcpy(&hb, bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(&hw, worst, 8, cudaMemcpyDeviceToHost);
  double w; memcpy(&w, &hw, 8);
  printf("%d %llu %.6f\n", (int)e, hb, w);
  return e == cudaSuccess ? 0 : 1;
}
"""


def test_logf_intrinsic_within_documented_error():
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.cu")
        exe = os.path.join(d, "probe")
        with open(src, "w") as f:
            f.write(PROBE.replace("#include <cmath>", "#include <cmath>\n#include <cstring>"))
        subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe, src])
        out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    status, bad, worst = out.stdout.split()
    assert out.returncode == 0 and status == "0", out.stdout
    assert int(bad) == 0, out.stdout
    assert float(worst) <= 1.0, out.stdout
