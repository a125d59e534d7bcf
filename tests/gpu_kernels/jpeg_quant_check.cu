// Exhaustive check of the JPEG quantiser division: dev::quotient_by(x, q, RN(1/q)) against
// __fdiv_rn(x, q) for every float x in [0.5, 2048) and every quantiser q in 1..255 (the DCT
// outputs of 8-bit samples stay below 1025 in magnitude; the division is odd in x, and below 0.5
// every quotient rounds to zero).  Built and run by tests/test_gpu_division.py; prints the mismatch
// count and exits non-zero on any mismatch.
#include <cstdio>

#include "../../im-operator_gb300/csrc/isp_device.cuh"

__global__ void check_quotients(unsigned lo, unsigned hi, unsigned long long* bad, unsigned* first) {
    for (unsigned bits = lo + blockIdx.x * blockDim.x + threadIdx.x; bits < hi; bits += gridDim.x * blockDim.x) {
        const float x = __uint_as_float(bits);
        unsigned n = 0;
        for (int q = 1; q <= 255; q++) {
            const float fq = (float)q, rq = __frcp_rn(fq);
            const float a = imop::dev::quotient_by(x, fq, rq), b = __fdiv_rn(x, fq);
            n += __float_as_uint(a) != __float_as_uint(b);
        }
        if (n) {
            atomicAdd(bad, n);
            atomicMin(first, bits);
        }
    }
}

int main() {
    const unsigned lo = 0x3f000000u, hi = 0x45000000u;  // 0.5f .. 2048.0f
    unsigned long long* bad = nullptr;
    unsigned* first = nullptr;
    if (cudaMalloc(&bad, sizeof(*bad)) || cudaMalloc(&first, sizeof(*first))) return 2;
    const unsigned init = 0xffffffffu;
    cudaMemset(bad, 0, sizeof(*bad));
    cudaMemcpy(first, &init, sizeof(init), cudaMemcpyHostToDevice);
    check_quotients<<<152 * 16, 256>>>(lo, hi, bad, first);
    unsigned long long nb = 0;
    unsigned f = 0;
    if (cudaMemcpy(&nb, bad, sizeof(nb), cudaMemcpyDeviceToHost) || cudaMemcpy(&f, first, sizeof(f), cudaMemcpyDeviceToHost))
        return 3;
    printf("jpeg quotients: %u values x 255 quantisers, %llu mismatches", hi - lo, nb);
    if (nb) printf(" (first x bits 0x%08x)", f);
    printf("\n");
    return nb ? 1 : 0;
}
