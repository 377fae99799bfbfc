/* qmetal_kernels.h -- the thin C-ABI layer between the C++ host and the
 * hand-written sm_103a kernels.
 *
 * Plain device pointers and sizes only; a CUDA stream travels as void*
 * (cudaStream_t). Every state pointer addresses 2^n complex64 amplitudes,
 * interleaved (re, im), LSB-first, 16-byte aligned. Matrices are row-major
 * 2x2 complex as 8 floats (re00, im00, re01, im01, re10, im10, re11, im11).
 * Every entry point returns 0 on success, a positive cudaError_t value when a
 * launch fails, or -1 for arguments it rejects (nothing is launched then).
 *
 * Each function names the reference kernel it replaces (file:line in the
 * reference project's src/metal/kernels.metal, and the host code that drove
 * it in src/metal/simulator.mm).
 */
#ifndef QMETAL_KERNELS_H
#define QMETAL_KERNELS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* |0...0>. Replaces init_basis (kernels.metal:39-44; simulator.mm:340-346). */
int qmk_init_basis(float *state, uint32_t n, void *stream);

/* 2x2 on wire q. Replaces apply_1q (kernels.metal:48-61; simulator.mm:453-463). */
int qmk_apply_1q(float *state, uint32_t n, uint32_t q, const float m[8],
                 void *stream);

/* Multiply every amplitude whose index has all `mask` bits set by
 * (re + i im); mask has 1..3 bits. Replaces apply_diagonal_2q
 * (kernels.metal:168-178; simulator.mm:388-402), and serves diag(1, e^{ia})
 * one-qubit gates at a quarter of the traffic of a dense 2x2. */
int qmk_apply_phase(float *state, uint32_t n, uint64_t mask, float re,
                    float im, void *stream);

/* k commuting 2x2s on distinct ascending wires in one pass: wire 0 pairs the
 * lanes of each vector, wires 1..5 exchange with partner lanes by warp
 * shuffle, wires >= 6 pair registers. One launch takes wire 0 plus up to five
 * wires in 1..5 and four wires >= 6 (k <= 10), or, with no wire in 1..5,
 * wire 0 plus up to five others. Replaces apply_1q_group{2,3,4}
 * (kernels.metal:71-102; simulator.mm:500-525). */
int qmk_apply_group(float *state, uint32_t n, uint32_t k,
                    const uint32_t *qubits, const float *matrices,
                    void *stream);

/* A run of `count` 2x2s on wires < block_bits applied in order to each
 * 2^block_bits block staged in shared memory; block_bits in 2..14.
 * Replaces apply_1q_blocked (kernels.metal:112-143; simulator.mm:464-499). */
int qmk_apply_blocked(float *state, uint32_t n, uint32_t block_bits,
                      uint32_t count, const uint32_t *qubits,
                      const float *matrices, void *stream);

/* 2x2 on `target` where every control bit is set; 1 or 2 controls (CX, CY,
 * CCX). Replaces apply_controlled_1q (kernels.metal:148-163;
 * simulator.mm:526-537) and apply_ccx (kernels.metal:392-408). */
int qmk_apply_controlled(float *state, uint32_t n, uint32_t num_controls,
                         const uint32_t *controls, uint32_t target,
                         const float m[8], void *stream);

/* Exchange |..1_a..0_b..> and |..0_a..1_b..>. Replaces apply_swap
 * (kernels.metal:181-194; simulator.mm:538-547). */
int qmk_apply_swap(float *state, uint32_t n, uint32_t a, uint32_t b,
                   void *stream);

/* A basis permutation affine over GF(2), out of place: dst[y] = src[G(y)]
 * with G(y) = offset ^ XOR of cols[j] over the set bits j of y (cols[j] is
 * the image of bit j; n entries, each non-zero and inside n bits, jointly
 * invertible). A run of CX / SWAP / X gates is such a map, so the run costs
 * one pass instead of one per gate; it replaces consecutive
 * apply_controlled_1q / apply_swap dispatches (simulator.mm:526-547) and has
 * no single counterpart there. The pass runs as that gather or as the
 * equivalent scatter through G^-1, whichever map spreads a warp's accesses
 * further. dst and src must not overlap. Returns -1 for a singular map or
 * bad arguments, without launching. */
int qmk_apply_permutation(float *dst, const float *src, uint32_t n,
                          const uint64_t *cols, uint64_t offset, void *stream);

/* Scratch bytes every workspace must hold for a simulator of n qubits (the
 * diagonal-layer tables and reduction partials). */
size_t qmk_workspace_bytes(uint32_t n);

/* Zero the workspace bookkeeping (call once after allocating it). */
int qmk_workspace_init(void *workspace, size_t bytes, void *stream);

/* amplitude i *= exp(i (global_phase + sum of angles[t] over terms whose mask
 * is fully set in i)), one pass. Phase sums are formed in FP64.
 * Replaces apply_diagonal_layer (kernels.metal:203-218; simulator.mm:559-592). */
int qmk_apply_diagonal(float *state, uint32_t n, uint32_t num_terms,
                       const uint64_t *masks, const double *angles,
                       double global_phase, void *workspace,
                       size_t workspace_bytes, void *stream);

/* Returned when a size exceeds a fixed capacity (nothing is launched). */
#define QMK_ERR_TOO_LARGE (-2)

/* qmk_apply_diagonal for callers that cannot allocate device memory; no
 * counterpart in the reference. Same arguments and result, minus the
 * workspace: the scratch is a 327 KiB file-scope device array that every GPU
 * loading this library holds until the process exits. Allocates nothing
 * (no cudaMalloc / cudaFree or any allocating routine). The first call on
 * each device looks up the array's device address (cudaGetSymbolAddress),
 * so make that first call before any stream capture. The address is kept
 * for the life of the process, so do not call this again on a device after
 * cudaDeviceReset in the same process (the reset drops the array with the
 * context). All calls share the array: calls whose kernels may overlap on
 * the GPU race. States above 34 qubits return QMK_ERR_TOO_LARGE. */
int qmk_apply_diagonal_noalloc(float *state, uint32_t n, uint32_t num_terms,
                               const uint64_t *masks, const double *angles,
                               double global_phase, void *stream);

/* sum |a_i|^2 into *d_out (device double). FP32 per-thread runs, FP64 from
 * the warp up, fixed-order final sum. Replaces reduce_abs2
 * (kernels.metal:250-268; simulator.mm:615-625). */
int qmk_abs2sum(const float *state, uint32_t n, double *d_out,
                void *workspace, size_t workspace_bytes, void *stream);

/* Terms sharing one flip mask (flip = x|y), up to 16 per call. d_out[t]
 * receives <psi|P_t|psi> for sign mask sign_masks[t] (= y|z) and Y count
 * ny[t]. Replaces reduce_pauli (kernels.metal:273-307; simulator.mm:629-661). */
int qmk_pauli_expect(const float *state, uint32_t n, uint64_t flip,
                     uint32_t num_terms, const uint64_t *sign_masks,
                     const uint32_t *ny, double *d_out, void *workspace,
                     size_t workspace_bytes, void *stream);

/* lambda (=|+=) sum_t coeff_t * i^ny_t * P_t psi over terms sharing one flip
 * mask, up to 16 per call; coeffs real. overwrite != 0 stores instead of
 * accumulating. Replaces pauli_accum + zero_state (kernels.metal:313-327,
 * 363-367; simulator.mm:856-895). */
int qmk_pauli_accum(float *lambda, const float *psi, uint32_t n,
                    uint64_t flip, uint32_t num_terms,
                    const uint64_t *sign_masks, const uint32_t *ny,
                    const double *coeffs, int overwrite, void *stream);

/* lambda (=|+=) sum_t coeff_t * i^ny_t * P_t psi for terms that each flip a
 * single wire (wires[t]; sign mask and Y count as for qmk_pauli_accum), up
 * to 16 per call, on wire 0, wires 1..5 and at most four wires >= 6, with
 * n >= 6 + that count: one pass over both states for all of them, where the
 * per-flip form takes one pass per wire (a transverse field on n wires is
 * n passes there). No counterpart in the reference, which builds the
 * co-state one term per pass (simulator.mm:856-895). */
int qmk_pauli_accum_local(float *lambda, const float *psi, uint32_t n,
                          uint32_t num_terms, const uint32_t *wires,
                          const uint64_t *sign_masks, const uint32_t *ny,
                          const double *coeffs, int overwrite, void *stream);

/* A transverse field: lambda (=|+=) sum_w coeffs[k] X_w psi over distinct
 * wires w = wires[k] (no Y, no Z signs), any of wires 0..5 and at most seven
 * wires >= 6, n >= 10: one pass over both states, psi staged through shared
 * memory. energy 1 writes, 2 adds, sum_k coeffs[k] <psi|X_w|psi> to
 * *d_energy (0: neither; the workspace is then not used). Refuses repeated
 * or out-of-range wires. No counterpart in the reference, which builds the
 * co-state one term per pass and the energy by a separate reduction
 * (simulator.mm:856-904). */
int qmk_xfield_costate(float *lambda, const float *psi, uint32_t n,
                       uint32_t num_wires, const uint32_t *wires,
                       const double *coeffs, int overwrite, double *d_energy,
                       int energy, void *workspace, size_t workspace_bytes,
                       void *stream);

/* Re<a|b> into *d_out. Replaces the host energy loop of simulator.mm:897-904. */
int qmk_dot_re(const float *a, const float *b, uint32_t n, double *d_out,
               void *workspace, size_t workspace_bytes, void *stream);

/* One backward step of the adjoint sweep for a one-qubit gate on wire q:
 * if generator is 1/2/3 (X/Y/Z), *d_grad = Im<lambda|P_q|psi> taken before
 * the undo; then minv (the gate's inverse) is applied to both psi and
 * lambda, in the same pass. generator 0 only undoes. Replaces reduce_pauli2
 * plus the two undo dispatches (kernels.metal:331-360; simulator.mm:914-959). */
int qmk_adjoint_1q(float *psi, float *lambda, uint32_t n, uint32_t q,
                   const float minv[8], int generator, double *d_grad,
                   void *workspace, size_t workspace_bytes, void *stream);

/* Co-state of a Hamiltonian of Z strings (each mask at most two bits):
 * lambda_i = D(i) psi_i with D(i) = sum_t c_t (-1)^{popcount(i & z_t)}, and
 * *d_energy = sum_i D(i) |psi_i|^2, in one pass. Returns -1 (nothing
 * launched) if a mask has three or more bits. Replaces the per-term
 * pauli_accum passes and the host energy loop for such Hamiltonians
 * (kernels.metal:313-327; simulator.mm:856-904). */
int qmk_zdiag_costate(float *lambda, const float *psi, uint32_t n, uint32_t num_terms,
                      const uint64_t *z_masks, const double *coeffs, double *d_energy,
                      void *workspace, size_t workspace_bytes, void *stream);

/* Backward step over a whole diagonal block (terms as in
 * qmk_apply_diagonal, describing the block's forward phases): for each of the
 * ngen <= 48 Z-string generators, d_grad[slots[t]] = Im<lambda|Z_gen|psi>;
 * then, if undo, both states are multiplied by the conjugate phases, all in
 * one pass. Replaces the per-gate reduce_pauli2 and undo dispatches for the
 * block's RZ gates and ZZ couplings (kernels.metal:331-360;
 * simulator.mm:914-959). */
int qmk_adjoint_diagonal(float *psi, float *lambda, uint32_t n, uint32_t num_terms,
                         const uint64_t *masks, const double *angles, double global_phase,
                         uint32_t ngen, const uint64_t *gen_masks, const uint32_t *slots,
                         double *d_grad, int undo, void *workspace, size_t workspace_bytes,
                         void *stream);

/* Backward step over a window tile of one-qubit gates, applied in the given
 * order (each wire's gates last to first): op o takes d_grad[slots[o]] =
 * Im<lambda|P|psi> if gens[o] is 1/2/3 (X/Y/Z), then applies
 * minv[8o..8o+7] to both states; one pass. From n >= 6 + h a tile holds wire
 * 0, any of wires 1..5 and h <= 4 wires >= 6, up to 32 ops of which up to 16
 * carry a gradient (20 in the tile of wire 0, wires 1..5 and four wires >= 6
 * where every wire carries RZ then RY); below that, wire 0 and up to three
 * wires >= 1 and 16 ops. A tile of five or six wires >= 6 and no other wire
 * is taken when every wire carries the same rotation sequence (one RX, RY or
 * RZ per wire, or RZ then RY, or RY then RZ). Returns -1 (nothing launched)
 * for any other shape. Replaces the
 * per-gate reduce_pauli2 and undo dispatches (kernels.metal:331-360;
 * simulator.mm:914-959). */
int qmk_adjoint_group(float *psi, float *lambda, uint32_t n, uint32_t num_ops,
                      const uint32_t *wires, const float *minv, const int *gens,
                      const uint32_t *slots, double *d_grad, void *workspace,
                      size_t workspace_bytes, void *stream);

/* How many bounded waits of the window-tile kernels that ran on `workspace`
 * gave up since the last call (each wait is on a bulk copy into shared
 * memory; one that gives up leaves that pass's results invalid), and reset
 * the count: a copy on `stream` and a synchronisation of it, so call it with
 * the stream that ran the passes. The count is the workspace's own, so
 * callers on separate workspaces never see each other's. 0, -1 (bad
 * arguments) or a CUDA error code. */
int qmk_take_wait_timeouts(void *workspace, size_t workspace_bytes, unsigned int *out,
                           void *stream);

/* Device address of that count inside `workspace` (a uint32 that
 * qmk_workspace_init zeroes and the passes only increase), for a caller that
 * reads it with its own asynchronous copy. */
unsigned int *qmk_wait_counter(void *workspace);

/* Fault injection for tests: the bounded bulk-copy waits inside the window
 * passes that run on `workspace` give up after `polls` polls (0: at once,
 * so the pass is counted as timed out and its results are invalid); a
 * negative value restores the full bound (2^22 polls). The wait each block
 * makes before it exits, for copies still in flight, always keeps the full
 * bound. Ordered on `stream`, which it synchronises. 0, -1 (bad arguments)
 * or a CUDA error code. */
int qmk_set_wait_poll_limit(void *workspace, size_t workspace_bytes, long long polls,
                            void *stream);

/* Sampling workspace bytes for n qubits (block CDF in FP64). */
size_t qmk_sample_workspace_bytes(uint32_t n);

/* Draw `shots` basis indices into d_out (device uint64) with the splitmix64
 * stream of `seed`: FP64 block sums over 1024-amplitude blocks, device prefix
 * scan, binary search per shot, warp walk inside the block. Replaces
 * block_abs2 and the host CDF/search/walk (kernels.metal:372-387;
 * simulator.mm:677-763). */
int qmk_sample(const float *state, uint32_t n, uint64_t shots, uint64_t seed,
               uint64_t *d_out, void *workspace, size_t workspace_bytes,
               void *stream);

#ifdef __cplusplus
}
#endif

#endif /* QMETAL_KERNELS_H */
