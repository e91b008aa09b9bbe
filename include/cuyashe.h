/*
 * cuyashe.h -- C ABI of the GB300-native (sm_103a) cuYASHE hot path.
 *
 * The reference crosses from host C++ into CUDA only through the static
 * launchers of `class CUDAFunctions` (src/cuda_functions.h:19-84) and the free
 * functions callCRT / callICRT / callCuModN (src/cuda_bn.h:76-87). Above them sit
 * `Polynomial` (src/polynomial.h), `Ciphertext` (src/ciphertext.h) and `Yashe`
 * (src/yashe.h). This header replaces that boundary with plain C: opaque
 * handles, caller-owned buffers, explicit streams, status codes.
 *
 * Data layout. A polynomial of a ring with N coefficients and modulus q is N
 * coefficients of L = ceil(bits(q)/64) little-endian uint64 limbs each
 * ([N][L]); a batch is [batch][N][L]. Inputs must lie in [0, q). The `d_`
 * prefix marks device pointers, `h_` host pointers.
 *
 * Errors. Every function returns a cy_status; none aborts or throws. The
 * reference asserts on every CUDA result and throws `const char*`
 * (src/polynomial.cpp:424,450; src/cuda_bn.cu:1145). cy_last_error() returns a
 * per-thread message for the last failure.
 *
 * Threading. A handle may be used from several threads as long as calls that
 * share a handle's internal workspace do not overlap on the GPU: calls on one
 * handle are ordered on the stream they are given; calls on different streams
 * need their own cy_workspace (cy_*_ws variants). The reference keeps all state
 * in process-wide statics (src/polynomial.h:35-41, src/cuda_functions.cu:23-38)
 * and always uses stream 0 (src/polynomial.h:1384-1387).
 */
#ifndef CUYASHE_GB300_H
#define CUYASHE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cy_status {
    CY_OK = 0,
    CY_ERR_INVALID_ARGUMENT = -1,
    CY_ERR_UNSUPPORTED = -2,
    CY_ERR_CUDA = -3,
    CY_ERR_OUT_OF_MEMORY = -4,
    CY_ERR_NOT_INVERTIBLE = -5,
    CY_ERR_NO_KEYS = -6,
    CY_ERR_TIMEOUT = -7,
    CY_ERR_BUSY = -8,
    CY_ERR_INTERNAL = -9
} cy_status;

/* A cudaStream_t; NULL means the legacy default stream. */
typedef void *cy_stream_t;

/* Limits of this build. */
#define CY_MAX_LOGN 14        /* N up to 16384 */
#define CY_MAX_Q_BITS 384     /* q up to 384 bits (6 limbs) */
#define CY_MAX_CRT_PRIMES 40  /* word-sized NTT primes per basis */

const char *cy_status_string(int status);
const char *cy_last_error(void);
int cy_version(void);

/* ------------------------------------------------------------------------ */
/* Rings Z_q[x]/(x^N+1)                                                      */
/* ------------------------------------------------------------------------ */

typedef struct cy_ring cy_ring;
typedef struct cy_yashe cy_yashe; /* declared with its functions below */
typedef struct cy_workspace cy_workspace;

typedef struct cy_ring_info {
    int n;              /* coefficients */
    int q_limbs;        /* 64-bit limbs per coefficient */
    int q_bits;
    int crt_primes;     /* primes of the product basis */
    int crt_bits;       /* bits of their product M */
    uint32_t primes[CY_MAX_CRT_PRIMES];
} cy_ring_info;

/* Builds the ring for N (power of two, 2..16384) and q < 2^384: picks the
 * word-sized NTT-friendly CRT basis with M > 4*N*q^2 (the reference's rule,
 * src/polynomial.h:914, is M >= 2*N*q^2), uploads twiddles and CRT/ICRT
 * constants. Replaces Polynomial::gen_crt_primes (src/polynomial.h:898-955),
 * CUDAFunctions::write_crt_primes (src/cuda_bn.cu:1047-1146) and
 * CUDAFunctions::init (src/cuda_functions.cu:878-956). The ring is bound to the
 * CUDA device current at creation. */
cy_status cy_ring_create(int n, const uint64_t *h_q, int q_limbs, cy_ring **out);
cy_status cy_ring_destroy(cy_ring *ring);
cy_status cy_ring_get_info(const cy_ring *ring, cy_ring_info *info);

/* Scratch for calls that run on different streams at the same time. A NULL
 * workspace means the ring's own (grown on demand with cudaMalloc). */
cy_status cy_workspace_create(cy_workspace **out);
cy_status cy_workspace_destroy(cy_workspace *ws);

/* c = a*b mod (x^N+1, q) for `batch` independent products.
 * Replaces `Polynomial c = a*b; c.reduce();` (src/polynomial.cpp:52-60,
 * src/common.h:136-226, src/cuda_functions.cu:617-738 and :1040-1077):
 * CRT split, forward NTTs, pointwise product, inverse NTT, ICRT and mod q all
 * run on the GPU. Asynchronous on `stream`. */
cy_status cy_polymul(cy_ring *ring, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_c, int batch,
                     cy_stream_t stream);
cy_status cy_polymul_ws(cy_ring *ring, cy_workspace *ws, const uint64_t *d_a, const uint64_t *d_b,
                        uint64_t *d_c, int batch, cy_stream_t stream);

/* Same product with host buffers; returns once h_c is written (the
 * reference's with-memcopy path, src/benchmark_polynomial.cpp:361-388). The
 * batch runs in chunks whose copies overlap the kernels of neighbouring chunks
 * when the buffers are page-locked; pageable buffers give the same result
 * without the overlap. */
cy_status cy_polymul_host(cy_ring *ring, const uint64_t *h_a, const uint64_t *h_b, uint64_t *h_c, int batch);

/* c = a + b mod q and c = a - b mod q, elementwise over the batch.
 * Replaces callPolynomialAddSub (src/cuda_functions.cu:99-165), which adds
 * residues without reduction. */
cy_status cy_polyadd(cy_ring *ring, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_c, int batch,
                     cy_stream_t stream);
cy_status cy_polysub(cy_ring *ring, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_c, int batch,
                     cy_stream_t stream);

/* c = s*a mod q for a scalar s in [0, q) given as q_limbs limbs.
 * Replaces Polynomial::operator*(ZZ) / callPolynomialOPInteger (MUL)
 * (src/polynomial.h:533-573, src/cuda_functions.cu:477-547). */
cy_status cy_poly_scalar_mul(cy_ring *ring, const uint64_t *d_a, const uint64_t *h_scalar, uint64_t *d_c,
                             int batch, cy_stream_t stream);

/* The product c = a*b mod (x^N+1, q), like cy_polymul, for callers that must
 * not allocate device memory: latency-critical or serving paths that cannot
 * take cudaMalloc's device-wide synchronisation, and hosts whose device memory
 * is owned by another allocator or admitted against a fixed budget. It calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch is a fixed
 * array of CY_NOALLOC_SCRATCH_BYTES in the library's device image, held by
 * every GPU that loads the library until the process exits.
 * Limit: batch * (CRT primes) * N * 4 bytes must fit in that array (at N = 4096
 * and a 127-bit q, 113 products per call), and batch <= 65535 (one launch);
 * larger batches are rejected with CY_ERR_INVALID_ARGUMENT and a message
 * giving the maximum. The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture. All calls share the array, so
 * calls that can overlap on the GPU race and must be serialised by the caller.
 * This entry point has no counterpart in the reference. */
#define CY_NOALLOC_SCRATCH_BYTES (16u << 20)
cy_status cy_polymul_noalloc(cy_ring *ring, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_c, int batch,
                             cy_stream_t stream);

/* Mixed batch: `njobs` products, each of its own ring (N and q may differ per
 * job). Products of rings with N in 1024..8192 and q up to 192 bits run in ONE
 * persistent launch that fuses CRT, forward NTTs, pointwise product, inverse
 * NTT, ICRT and mod q over a work list (largest transforms first, epilogue
 * units after the NTT units of their job); products of other rings go through
 * the per-ring path in the same call. The reference multiplies one pair per
 * call and re-initialises its tables whenever N changes (src/common.h:136-226).
 * Asynchronous on `stream`; calls on different streams are ordered on the
 * device by the library (they share one scratch per device). */
typedef struct cy_polymul_job {
    cy_ring *ring;
    const uint64_t *d_a;
    const uint64_t *d_b;
    uint64_t *d_c;
} cy_polymul_job;
cy_status cy_polymul_batched(const cy_polymul_job *jobs, int njobs, cy_stream_t stream);

/* Synchronises `stream` with the last mixed launch on this device and reports
 * CY_ERR_TIMEOUT if a block of it gave up waiting for its job's transforms (a
 * bounded wait that cannot expire unless the device stops making progress). */
cy_status cy_polymul_batched_status(cy_stream_t stream);

/* Prepared mixed batch: a fixed list of polynomial products and YASHE
 * multiplies (with or without relinearisation) of rings of different N
 * (1024..8192) and q (up to 192 bits), run as ONE persistent launch: per job
 * CRT split, forward NTTs, pointwise product, inverse NTT, ICRT with mod q (or
 * the YASHE rounding round(t/q .)), then for relinearised jobs the word
 * decomposition, NTT-domain product with the resident evaluation key, inverse
 * NTT and mod q, all in one kernel over a work list in dependency order.
 * cy_mixed_plan_create sizes and uploads everything (it allocates and
 * synchronises); cy_mixed_plan_launch then issues one memset and one kernel on
 * `stream`, with no allocation and no host synchronisation, so that a caller can
 * replay it freely (or record it: cy_mixed_plan_graph_create). Results equal
 * cy_polymul / cy_yashe_mul of each job alone, bit for bit. Outputs must not be
 * any job's inputs; launches of one plan must not overlap on the GPU (they share
 * the plan's scratch). The reference multiplies one pair per call and
 * re-initialises its tables whenever N changes (src/common.h:136-226); its
 * homomorphic multiply is a chain of such calls (src/ciphertext.cpp:38-130). */
typedef struct cy_mixed_job {
    cy_ring *ring;      /* a polynomial product in this ring, or NULL */
    cy_yashe *yashe;    /* a YASHE multiply of this scheme (keys set), or NULL */
    int relin;          /* YASHE: relinearise the product */
    const uint64_t *d_a, *d_b;  /* [N][L] operands (ciphertexts for YASHE) */
    uint64_t *d_c;      /* [N][L] result */
} cy_mixed_job;
typedef struct cy_mixed_plan cy_mixed_plan;
cy_status cy_mixed_plan_create(const cy_mixed_job *jobs, int njobs, cy_mixed_plan **out);
cy_status cy_mixed_plan_destroy(cy_mixed_plan *plan);
cy_status cy_mixed_plan_launch(cy_mixed_plan *plan, cy_stream_t stream);
/* Synchronises `stream` and reports CY_ERR_TIMEOUT if a block of the last
 * launch gave up waiting for earlier units of its job (a bounded wait that does
 * not expire while the device makes progress). */
cy_status cy_mixed_plan_status(cy_mixed_plan *plan, cy_stream_t stream);
/* Schedules of the mixed kernel: 0 = 8 coefficients per thread in 1024-thread
 * blocks, 1 = 16 per thread in 512-thread blocks. The autotuner runs each on the
 * plan's own buffers (results must agree bit for bit), times it with CUDA
 * events and keeps the fastest; it synchronises. */
cy_status cy_mixed_plan_set_schedule(cy_mixed_plan *plan, int schedule);
cy_status cy_mixed_plan_get_schedule(const cy_mixed_plan *plan, int *schedule);
cy_status cy_mixed_plan_autotune(cy_mixed_plan *plan, cy_stream_t stream);
/* For tests of the bounded wait only: makes the first epilogue of job `job`
 * wait for one more transform than the job has, so that its wait expires after
 * `spin_limit` back-off steps (about 0.3 us each) and the launch reports
 * CY_ERR_TIMEOUT through cy_mixed_plan_status. The plan's results are invalid
 * afterwards. No counterpart in the reference (it has no failure handling). */
cy_status cy_mixed_plan_test_starve(cy_mixed_plan *plan, int job, unsigned spin_limit);

/* Forward / inverse negacyclic NTT of residue vectors: d_res is [batch][k][N]
 * uint32 residues modulo the ring's CRT primes, transformed in place (values
 * in [0, p) on input and output; forward output in bit-reversed order, inverse
 * output scaled by N^-1). Replaces CUDAFunctions::callNTT
 * (src/cuda_functions.cu:447-458). */
cy_status cy_ntt(cy_ring *ring, uint32_t *d_res, int batch, int inverse, cy_stream_t stream);

/* Status of the standalone NTT's bounded waits: the N = 4096 schedule whose
 * inverse takes its input tile by TMA waits for each tile on a barrier with a
 * poll limit, and a block that gives up records CY_ERR_TIMEOUT on the device. This synchronises
 * the device, returns CY_ERR_TIMEOUT if any launch since the last call gave up
 * (with cy_last_error saying so) and clears the record. No counterpart in the
 * reference (it has no failure handling). */
cy_status cy_ntt_check(void);

/* Testing hook for that path: the next TMA inverse transforms poll at most
 * spin_limit times (0: the default) and tell the tile's barrier to expect
 * extra_bytes beyond the tile (0: none; > 0 makes every wait run out). */
cy_status cy_ntt_test_wait(unsigned spin_limit, unsigned extra_bytes);

/* CRT split and ICRT recombination on their own (callCRT / callICRT,
 * src/cuda_bn.cu:970-1045): d_res [batch][k][N] uint32 <-> d_x [batch][N][L]. */
cy_status cy_crt(cy_ring *ring, const uint64_t *d_x, uint32_t *d_res, int batch, cy_stream_t stream);
cy_status cy_icrt(cy_ring *ring, const uint32_t *d_res, uint64_t *d_x, int batch, cy_stream_t stream);

/* ------------------------------------------------------------------------ */
/* YASHE (Bos, Lauter, Loftus, Naehrig 2013)                                 */
/* ------------------------------------------------------------------------ */

typedef struct cy_yashe cy_yashe;

typedef struct cy_yashe_params {
    int n;               /* ring degree N */
    const uint64_t *q;   /* ciphertext modulus, q_limbs limbs, odd */
    int q_limbs;
    uint64_t t;          /* plaintext modulus, 2 <= t < 2^32 */
    int w_bits;          /* relinearisation digit width; 32 */
    double sigma;        /* error parameter of the discrete Gaussian (8.0) */
} cy_yashe_params;

typedef struct cy_yashe_info {
    int n, q_limbs, q_bits, ell, w_bits;
    uint64_t t;
    int tensor_primes;   /* CRT basis of the tensor product */
    int relin_primes;    /* CRT basis of the keyswitch */
    int has_keys;
} cy_yashe_info;

/* Replaces the statics Yashe::{d,q,t,w,lwq} (src/yashe.h:17-29) and their set-up
 * in the reference's fixtures (src/test.cu:73-133). */
cy_status cy_yashe_create(const cy_yashe_params *params, cy_yashe **out);
cy_status cy_yashe_destroy(cy_yashe *y);
cy_status cy_yashe_get_info(const cy_yashe *y, cy_yashe_info *info);
cy_status cy_yashe_get_ring(cy_yashe *y, cy_ring **ring);

/* Key generation on the host (set-up time): f = t*f'+1 with ternary f', real
 * f^-1 in R_q, h = [t*g*f^-1]_q, evk_d = [f*w^d + e_d + h*s_d]_q. The evaluation
 * key is then kept resident on the GPU in the NTT domain. Replaces
 * Yashe::generate_keys (src/yashe.cpp:17-102), which stubs f^-1 with f. */
cy_status cy_yashe_keygen(cy_yashe *y, uint64_t seed);

/* Installs externally generated keys (host arrays): f [N][L], h [N][L],
 * evk [ell][N][L]. */
cy_status cy_yashe_set_keys(cy_yashe *y, const uint64_t *h_f, const uint64_t *h_h, const uint64_t *h_evk);
cy_status cy_yashe_get_keys(const cy_yashe *y, uint64_t *h_f, uint64_t *h_h, uint64_t *h_evk);

/* c = [Delta*m + e + h*s]_q on the host (set-up time); m: [batch][N] uint64 in
 * [0, t); ct: [batch][N][L]. Replaces Yashe::encrypt (src/yashe.cpp:104-142). */
cy_status cy_yashe_encrypt_host(cy_yashe *y, const uint64_t *h_m, uint64_t *h_ct, int batch, uint64_t seed);

/* Encryption on the GPU: ct = [h*s + e + Delta*(m mod t)]_q, Delta = floor(q/t),
 * with s and e drawn on the GPU from the discrete Gaussian of width sigma on
 * [-B, B], B = ceil(6 sigma). Draw c of a call is the c-th output of
 * splitmix64 seeded with `seed` (mix(seed + (c+1) * 0x9E3779B97F4A7C15));
 * coefficient i of s (of e) of ciphertext b uses c = 2b*N + i ((2b+1)*N + i),
 * mapped through the 64-bit CDT thresholds T_j = floor(2^64 * sum_{x<=j-B}
 * w_x / sum w), w_x = exp(-x^2 / (2 sigma^2)), to the first j with draw < T_j.
 * d_m: [batch][N] uint64; d_ct: [batch][N][L]. Asynchronous on `stream`.
 * Replaces Yashe::encrypt and its samplers (src/yashe.cpp:104-142,
 * src/distribution.cpp:4-60, src/cuda_distribution.cu:11-35). */
cy_status cy_yashe_encrypt(cy_yashe *y, const uint64_t *d_m, uint64_t *d_ct, int batch, uint64_t seed,
                           cy_stream_t stream);

/* The CDT thresholds T_0 .. T_{2B} that cy_yashe_encrypt uses for width sigma
 * (host only, no GPU). *n_entries is set to 2B+1; fails if it exceeds
 * max_entries. No counterpart in the reference, whose sampler is cuRAND. */
cy_status cy_gaussian_cdt(double sigma, uint64_t *out, int max_entries, int *n_entries);

/* m = [round(t/q * [key*c]_q)]_t on the GPU for every coefficient; key = f, or
 * f^2 when `aftermul` (a product that was not relinearised). m: [batch][N]
 * uint64. Replaces Yashe::decrypt (src/yashe.cpp:143-201), which decrypts
 * coefficient 0 only. */
cy_status cy_yashe_decrypt(cy_yashe *y, const uint64_t *d_ct, uint64_t *d_m, int batch, int aftermul,
                           cy_stream_t stream);

/* The YASHE rounding round(t/q * x) is first estimated in 64-bit fixed point
 * and computed exactly only for the rare coefficients (about one in 2^28) the
 * estimate cannot decide; both give the same result. on != 0 makes every
 * coefficient take the exact path (a check of the estimate; slower). Applies
 * to calls made after it, process-wide. No counterpart in the reference. */
cy_status cy_set_epilogue_exact(int on);

/* The ICRT epilogue has kernels specialised for the prime counts of common
 * parameter sets (their basis constants passed by value); on != 0 makes every
 * call use the generic kernel instead (a cross-check; slower). Results are
 * identical. Process-wide, for calls made after it; default off. No counterpart
 * in the reference. */
cy_status cy_set_epilogue_generic(int on);

/* Calls of several chunks run their chunks on two streams (the caller's and a
 * side stream of the workspace, with a second residue scratch) so that their
 * kernels overlap; on == 0 runs them one after another on the caller's stream
 * (less device memory; clean per-kernel timings). Results are identical.
 * Process-wide, for calls made after it; default on. No counterpart in the
 * reference. */
cy_status cy_set_chunk_overlap(int on);

/* Homomorphic multiply: out = [round(t/q * c1*c2)]_q with the product over
 * Z[x]/(x^N+1) on symmetric representatives, then (relin != 0) the keyswitch
 * [sum_d D_d(out)*evk_d]_q. Replaces Ciphertext::operator* and
 * Ciphertext::convert/keyswitch (src/ciphertext.cpp:38-130). */
cy_status cy_yashe_mul(cy_yashe *y, const uint64_t *d_c1, const uint64_t *d_c2, uint64_t *d_out, int batch,
                       int relin, cy_stream_t stream);
cy_status cy_yashe_mul_ws(cy_yashe *y, cy_workspace *ws, const uint64_t *d_c1, const uint64_t *d_c2,
                          uint64_t *d_out, int batch, int relin, cy_stream_t stream);

/* cy_yashe_mul on HOST buffers c1, c2, out ([batch][N][L] limbs); returns once
 * out is written. The batch runs in chunks whose host<->device copies overlap
 * the kernels of neighbouring chunks when the buffers are page-locked
 * (cudaHostAlloc / cudaHostRegister); pageable buffers give the same result
 * without the overlap. Replaces Ciphertext::operator* on host-resident
 * operands, i.e. update_device_data, the product and update_host_data
 * (src/ciphertext.cpp:38-73, src/polynomial.cpp:265-417). Calls on one device
 * share one pipeline and run one after another. */
cy_status cy_yashe_mul_host(cy_yashe *y, const uint64_t *h_c1, const uint64_t *h_c2, uint64_t *h_out, int batch,
                            int relin);

/* Relinearisation alone: out = [sum_d D_d(c)*evk_d]_q (Ciphertext::convert). */
cy_status cy_yashe_keyswitch(cy_yashe *y, const uint64_t *d_c, uint64_t *d_out, int batch, cy_stream_t stream);

/* Plaintext operations. add_plain: out = [c + Delta*(m mod t)]_q, the scheme's
 * addition of a plaintext (the reference's Ciphertext::operator+(Polynomial),
 * src/ciphertext.cpp:11-15, adds a polynomial that the caller has already
 * scaled; cy_polyadd does that). mul_plain: out = [c * m_c]_q with m_c the
 * representative of m mod t in (-t/2, t/2], which decrypts to the product of
 * the plaintexts mod t; no counterpart in the reference. d_m: [batch][N]
 * uint64; out must not alias c for mul_plain. Asynchronous on `stream`. */
cy_status cy_yashe_add_plain(cy_yashe *y, const uint64_t *d_c, const uint64_t *d_m, uint64_t *d_out, int batch,
                             cy_stream_t stream);
cy_status cy_yashe_mul_plain(cy_yashe *y, const uint64_t *d_c, const uint64_t *d_m, uint64_t *d_out, int batch,
                             cy_stream_t stream);

/* Homomorphic add (Ciphertext::operator+, src/ciphertext.cpp:4-23). */
cy_status cy_yashe_add(cy_yashe *y, const uint64_t *d_c1, const uint64_t *d_c2, uint64_t *d_out, int batch,
                       cy_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Wire / on-disk format for keys and ciphertexts (host only, no GPU)         */
/*                                                                            */
/* The reference has no serialised form (keys and ciphertexts are NTL objects */
/* in process memory). A blob is: magic "CYSH", u32 version (1), u32 kind,    */
/* u32 n, u32 q_limbs L, u32 count, u64 t, u32 w_bits, u32 reserved, q as L   */
/* u64, the polynomials [count][n][L] u64 (coefficients in [0, q)), and a u64 */
/* FNV-1a checksum of every preceding byte; all little endian.                */

#define CY_BLOB_CIPHERTEXTS 1u
#define CY_BLOB_PUBLIC_KEY 2u
#define CY_BLOB_SECRET_KEY 3u
#define CY_BLOB_EVAL_KEY 4u
#define CY_BLOB_KEYS 5u /* f, h, evk_0 .. evk_{ell-1} */
#define CY_BLOB_MAX_LIMBS 12

typedef struct cy_blob_info {
    uint32_t kind;
    int n, q_limbs, count, w_bits;
    uint64_t t;
    uint64_t q[CY_BLOB_MAX_LIMBS];
    size_t bytes; /* total size of the blob */
} cy_blob_info;

/* Writes a blob of `count` polynomials into buf (len bytes); *needed gets its
 * size. buf == NULL only reports the size. Rejects coefficients >= q. */
cy_status cy_serialize(uint32_t kind, int n, const uint64_t *q, int q_limbs, uint64_t t, int w_bits,
                       const uint64_t *polys, int count, void *buf, size_t len, size_t *needed);
/* Reads and checks a blob's header and checksum. */
cy_status cy_blob_info_read(const void *buf, size_t len, cy_blob_info *info);
/* Copies a checked blob's polynomials (count*n*q_limbs words) to polys. */
cy_status cy_deserialize(const void *buf, size_t len, uint64_t *polys, size_t max_words);

/* The keys of a scheme as one CY_BLOB_KEYS blob, and back (the parameters in
 * the blob must equal the scheme's). With a serving process these save its
 * resident keys and resume with them. */
cy_status cy_yashe_save_keys(const cy_yashe *y, void *buf, size_t len, size_t *needed);
cy_status cy_yashe_load_keys(cy_yashe *y, const void *buf, size_t len);

/* ------------------------------------------------------------------------ */
/* Serving: continuous batching of HE multiplies                              */
/* ------------------------------------------------------------------------ */

/* A request loop on the current device. A dispatcher thread admits pending
 * requests into batches of one registered YASHE context and one relin flag
 * (oldest request's first, FIFO within them, at most max_batch per batch) whenever one of
 * `streams` slots is free and device_budget_bytes has room for the batch's
 * inputs, outputs and scratch; batches of different contexts run concurrently
 * on different streams while new requests keep arriving. Evaluation keys stay
 * resident in each cy_yashe. Requests carry host buffers (read when the batch
 * is formed, written before the request completes; keep them alive until
 * cy_server_wait returns). Per-request latency (submit to completion) and
 * throughput are kept for cy_server_get_stats. The reference has no serving layer:
 * each Ciphertext::operator* runs alone and synchronises the device
 * (src/ciphertext.cpp:38-73, src/common.h:223). */
typedef struct cy_server cy_server;
typedef struct cy_server_config {
    size_t device_budget_bytes;  /* admission budget for in-flight batches */
    int streams;                 /* batches in flight at once (1..32) */
    int max_batch;               /* requests per batch */
    int poll_us;                 /* dispatcher poll period while batches run (default 20) */
    int batch_budget_us;         /* > 0: a batch of a context takes at most as many requests as fit
                                    this much GPU time, from a running estimate of the context's
                                    time per request (0: max_batch only) */
} cy_server_config;
typedef struct cy_serve_request {
    int class_id;                /* from cy_server_register */
    int relin;                   /* relinearise the product */
    const uint64_t *h_c1, *h_c2; /* [N][L] ciphertexts of the class's ring */
    uint64_t *h_out;             /* [N][L] result */
} cy_serve_request;
typedef struct cy_server_stats {
    uint64_t completed, rejected, failed, batches;
    double p50_us, p99_us, mean_us, throughput_per_s;
    size_t peak_device_bytes;
} cy_server_stats;

cy_status cy_server_create(const cy_server_config *cfg, cy_server **out);
cy_status cy_server_destroy(cy_server *server);
/* Registers a context that has keys; its requests form their own batches. */
cy_status cy_server_register(cy_server *server, cy_yashe *y, int *class_id);
/* Queues a request. Invalid requests (unknown class, NULL buffers) and requests
 * larger than the whole budget are rejected here and counted. */
cy_status cy_server_submit(cy_server *server, const cy_serve_request *req, uint64_t *ticket);
/* Requests on ciphertexts resident in device memory: the caller uploads them
 * once (or keeps the results of earlier requests) and names them by device
 * pointer. A batch of such requests is gathered on the device into the slot's
 * buffers, multiplied, and each product written to its d_out, with no host copy
 * in either direction; d_out stays on the device for the caller's next
 * operation. Buffers are 16-byte aligned device memory of the server's device,
 * [N][L] limbs of the class's ring; keep them alive and unchanged until the
 * request completes. `n` requests are queued in one call (tickets[i] for
 * reqs[i]); a rejected request stops the call at that index with its error, the
 * ones before it stay queued. Device requests batch apart from host-buffer ones.
 * The reference keeps each Polynomial's device copy between operations
 * (src/polynomial.cpp:265-340) but has no request loop. */
typedef struct cy_serve_request_dev {
    int class_id;                /* from cy_server_register */
    int relin;                   /* relinearise the product */
    const uint64_t *d_c1, *d_c2; /* [N][L] ciphertexts in device memory */
    uint64_t *d_out;             /* [N][L] result in device memory */
} cy_serve_request_dev;
cy_status cy_server_submit_device(cy_server *server, const cy_serve_request_dev *reqs, int n, uint64_t *tickets);
cy_status cy_server_poll(cy_server *server, uint64_t ticket, int *done);
/* Waits up to timeout_ms; returns the request's status (and forgets the ticket)
 * or CY_ERR_TIMEOUT (the request stays queued or running). */
cy_status cy_server_wait(cy_server *server, uint64_t ticket, int timeout_ms);
/* Waits until nothing is pending or running (CY_ERR_TIMEOUT at the deadline). */
cy_status cy_server_drain(cy_server *server, int timeout_ms);
cy_status cy_server_get_stats(cy_server *server, cy_server_stats *stats);
cy_status cy_server_reset_stats(cy_server *server);

/* ------------------------------------------------------------------------ */
/* CUDA graphs                                                                */
/* ------------------------------------------------------------------------ */

/* A fixed batch (fixed buffers) recorded once as a CUDA graph and replayed with
 * cy_graph_launch: one graph launch instead of one launch per kernel and chunk.
 * Creation runs the operation once (to size the graph's own workspace), then
 * captures it on a private stream; it synchronises. Replays of one graph must
 * not overlap each other on the GPU. The reference synchronises the device
 * after every operation (src/common.h:223). */
typedef struct cy_graph cy_graph;
cy_status cy_polymul_graph_create(cy_ring *ring, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_c, int batch,
                                  cy_graph **out);
cy_status cy_yashe_mul_graph_create(cy_yashe *y, const uint64_t *d_c1, const uint64_t *d_c2, uint64_t *d_out,
                                    int batch, int relin, cy_graph **out);
/* A prepared mixed batch (cy_mixed_plan_launch with the plan's current
 * schedule) recorded as a graph; the plan must outlive the graph. */
cy_status cy_mixed_plan_graph_create(cy_mixed_plan *plan, cy_graph **out);
cy_status cy_graph_launch(cy_graph *graph, cy_stream_t stream);
cy_status cy_graph_destroy(cy_graph *graph);

/* ------------------------------------------------------------------------ */
/* Schedule autotuning                                                        */
/* ------------------------------------------------------------------------ */

/* Each transform length is compiled with one or more NTT schedules (8 or 16
 * coefficients per thread: 512 or 256 threads per transform and 4 or 3
 * register passes at N = 4096). cy_ring_autotune runs every schedule of the
 * ring's product on `batch` synthetic jobs, requires each output to equal the
 * default schedule's bit for bit, and keeps the fastest for this device, N and
 * limb count; cy_yashe_autotune does the same for the plain product, the YASHE
 * tensor and the keyswitch. Synchronous; allocates its test buffers. The
 * reference has one fixed launch shape per kernel (src/cuda_functions.cu:447-458)
 * and hand-timed block sizes in comments (src/cuda_bn.cu:983-988). */
cy_status cy_ring_autotune(cy_ring *ring, int batch, cy_stream_t stream);
cy_status cy_yashe_autotune(cy_yashe *y, int batch, cy_stream_t stream);

/* The current device's choices as text, e.g. "n4096.l2.mul=1;n4096.l2.ks=0;"
 * (*needed gets the size including the terminator), and back. */
cy_status cy_tuning_export(char *buf, size_t len, size_t *needed);
cy_status cy_tuning_import(const char *spec);

/* ------------------------------------------------------------------------ */
/* Observability                                                              */
/* ------------------------------------------------------------------------ */

/* Kernels launched by this library since the process started. The reference
 * has no launch accounting; its timing is rdtsc/clock_gettime around whole
 * operations (src/common.cpp:15-59). */
uint64_t cy_launch_count(void);

/* Per-kernel tracing: between cy_trace_start and cy_trace_stop every launch is
 * bracketed by CUDA events recorded on the launch stream. cy_trace_stop
 * synchronises those events and returns, per kernel name, the number of
 * launches and the summed device time. Tracing adds two event records per
 * launch; leave it off in timed regions. */
typedef struct cy_trace_entry {
    char name[48];
    int launches;
    double total_ms;
} cy_trace_entry;
cy_status cy_trace_start(void);
cy_status cy_trace_stop(cy_trace_entry *entries, int max_entries, int *n_entries);

#ifdef __cplusplus
}
#endif

#endif /* CUYASHE_GB300_H */
