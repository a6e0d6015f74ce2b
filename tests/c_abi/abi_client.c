/*
 * A plain C client of include/kbwg.h: what a non-Python host (the Rust
 * QuantumExecution shim, a C plugin) does through the ABI, with no Python,
 * torch or CUDA headers involved.  Built and run by tests/test_c_client.py.
 *
 *   abi_client --no-gpu   checks the library links and fails cleanly
 *                         without a GPU (status codes, no crash)
 *   abi_client            runs on cuda:0: Bell and GHZ states through the
 *                         trait-style gate calls, measure_p1, dump, sample,
 *                         exp_value, sequential measurement, the error
 *                         paths, and the whole-circuit batch entry
 *
 * Exit status 0 on success; every failed check prints one line.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "kbwg.h"

static int failures = 0;

#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            failures++;                           \
            printf("FAIL %s:%d: ", __FILE__, __LINE__); \
            printf(__VA_ARGS__);                  \
            printf("\n");                         \
        }                                         \
    } while (0)

#define OK(call) CHECK((call) == KBWG_OK, "%s -> %s", #call, kbwg_last_error())

static int no_gpu(void) {
    const uint8_t *msg = NULL;
    uintptr_t len = 0;
    OK(kbwg_build_info(&msg, &len));
    CHECK(len > 0 && memcmp(msg, "kbw-gb300", 9) == 0, "build info");
    kbwg_sim *sim = (kbwg_sim *)0x1;
    CHECK(kbwg_new(41, KBWG_C64, 0, &sim) == KBWG_EQUBITS && sim == NULL, "41 qubits must be EQUBITS");
    sim = (kbwg_sim *)0x1;
    int32_t rc = kbwg_new(4, KBWG_C128, 0, &sim);
    CHECK(rc != KBWG_OK && sim == NULL, "kbwg_new without a GPU must fail cleanly (rc %d)", (int)rc);
    CHECK(strlen(kbwg_last_error()) > 0, "an error text is set");
    CHECK(kbwg_free(NULL) == KBWG_OK, "free(NULL)");
    return failures;
}

static void bell_and_ghz(int32_t prec, uint32_t flags) {
    const double tol = prec == KBWG_C128 ? 1e-12 : 1e-6;
    kbwg_sim *sim = NULL;
    OK(kbwg_new(20, prec, flags, &sim));
    if (!sim) return;
    /* GHZ on 20 qubits: H(0), then CNOT(q-1 -> q) */
    OK(kbwg_hadamard(sim, 0, NULL, 0));
    for (uintptr_t q = 1; q < 20; q++) {
        const uintptr_t c = q - 1;
        OK(kbwg_pauli_x(sim, q, &c, 1));
    }
    double p1 = 0.0;
    OK(kbwg_measure_p1(sim, 19, &p1));
    CHECK(fabs(p1 - 0.5) < tol, "GHZ p1(19) = %.17g", p1);
    /* dump of (19, 0): two entries, 0b00 and 0b11, amplitude 1/sqrt(2) */
    const uintptr_t dq[2] = {19, 0};
    uint64_t st[4];
    double re[4], im[4];
    uintptr_t size = 0;
    OK(kbwg_dump(sim, dq, 2, st, re, im, 4, &size));
    CHECK(size == 2 && st[0] == 0 && st[1] == 3, "GHZ dump support (size %lu)", (unsigned long)size);
    CHECK(fabs(re[0] - 0.70710678118654752440) < tol && fabs(re[1] - 0.70710678118654752440) < tol && fabs(im[0]) < tol, "GHZ amplitudes");
    /* <Z0 Z19> = 1, <X0> = 0 */
    const uint8_t paulis[3] = {KBWG_PAULI_Z, KBWG_PAULI_Z, KBWG_PAULI_X};
    const uintptr_t pq[3] = {0, 19, 0};
    const uintptr_t off[3] = {0, 2, 3};
    const double coef[2] = {1.0, 0.25};
    double e = 0.0;
    OK(kbwg_exp_value(sim, paulis, pq, off, coef, 2, &e));
    CHECK(fabs(e - 1.0) < tol, "<Z0 Z19> + 0.25 <X0> = %.17g", e);
    /* 1000 samples of (19, 0) with draws below / above 1/2 */
    double draws[1000];
    for (int i = 0; i < 1000; i++) draws[i] = (i % 2) ? 0.75 : 0.25;
    uint64_t ss[4], sc[4];
    uintptr_t nout = 0;
    OK(kbwg_sample(sim, dq, 2, 1000, draws, ss, sc, 4, &nout));
    CHECK(nout == 2 && ss[0] == 0 && ss[1] == 3 && sc[0] == 500 && sc[1] == 500, "GHZ sample histogram");
    /* sequential measurement: all 20 qubits agree */
    uintptr_t all[20];
    double md[20];
    for (int q = 0; q < 20; q++) {
        all[q] = (uintptr_t)q;
        md[q] = 0.9;
    }
    uint64_t bits = 0;
    OK(kbwg_measure(sim, all, 20, md, &bits));
    CHECK(bits == 0 || bits == 0xFFFFFull, "GHZ measurement 0x%llx", (unsigned long long)bits);
    /* error paths are status codes */
    const uintptr_t bad = 20;
    CHECK(kbwg_pauli_x(sim, 20, NULL, 0) == KBWG_EINVAL, "target out of range");
    CHECK(kbwg_pauli_x(sim, 3, &bad, 1) == KBWG_EINVAL, "control out of range");
    CHECK(kbwg_dump(sim, dq, 2, st, re, im, 0, &size) == KBWG_ECAPACITY && size >= 1, "dump capacity query");
    OK(kbwg_free(sim));
}

static void batch_entry(void) {
    /* Bell pair through BatchExecution-style exp_value: <Z0 Z1> = 1, <X0 X1> = 1 */
    const kbwg_gate gates[2] = {{KBWG_H, 0, 0, 0.0}, {KBWG_X, 1, 1ull << 0, 0.0}};
    const uint8_t paulis[4] = {KBWG_PAULI_Z, KBWG_PAULI_Z, KBWG_PAULI_X, KBWG_PAULI_X};
    const uintptr_t pq[4] = {0, 1, 0, 1};
    const uintptr_t off[3] = {0, 2, 4};
    const double coef[2] = {1.0, 1.0};
    const uintptr_t ham_off[3] = {0, 1, 2};
    double out[2] = {0.0, 0.0};
    OK(kbwg_batch_exp_value(14, KBWG_C128, KBWG_FLAG_FAST_C128, gates, 2, paulis, pq, off, coef, ham_off, 2, out));
    CHECK(fabs(out[0] - 1.0) < 1e-12 && fabs(out[1] - 1.0) < 1e-12, "batch <ZZ>, <XX> = %.17g %.17g", out[0], out[1]);
    OK(kbwg_batch_release());
}

int main(int argc, char **argv) {
    if (argc > 1 && strcmp(argv[1], "--no-gpu") == 0) {
        no_gpu();
    } else {
        bell_and_ghz(KBWG_C128, 0);
        bell_and_ghz(KBWG_C128, KBWG_FLAG_FAST_C128);
        bell_and_ghz(KBWG_C64, 0);
        batch_entry();
    }
    printf("%s (%d failures)\n", failures ? "FAILED" : "ok", failures);
    return failures ? 1 : 0;
}
