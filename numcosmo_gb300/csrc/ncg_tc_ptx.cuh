/*
 * ncg_tc_ptx.cuh -- inline-PTX helpers for the tcgen05 kernels (ncg_eval_tc.cu,
 * ncg_syrk_tc.cu): mbarriers with bounded waits, bulk copies, shared-memory
 * matrix descriptors (K-major, no swizzle), MMA commit, TMEM loads, TF32
 * rounding and the core-matrix layout.
 *
 * Operand layout used by both kernels: K-major, no swizzle, 8-row x 16-byte
 * core matrices, K-chunk outermost: element (row, k) of a tile with R rows
 * sits at byte (k / 4) * LBO + (row / 8) * 128 + (row % 8) * 16 + (k % 4) * 4,
 * LBO = R / 8 * 128 (the descriptor's leading byte offset), SBO = 128.
 */
#ifndef NCG_TC_PTX_CUH
#define NCG_TC_PTX_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#define TC_SBO 128


static __device__ __forceinline__ uint32_t
_smem_u32 (const void *p)
{
  return (uint32_t) __cvta_generic_to_shared (p);
}

static __device__ __forceinline__ void
_mbar_init (uint64_t *bar, uint32_t count)
{
  asm volatile ("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(_smem_u32 (bar)), "r"(count) : "memory");
}

static __device__ __forceinline__ void
_mbar_arrive (uint64_t *bar)
{
  asm volatile ("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(_smem_u32 (bar)) : "memory");
}

static __device__ __forceinline__ void
_mbar_arrive_tx (uint64_t *bar, uint32_t bytes)
{
  asm volatile ("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(_smem_u32 (bar)), "r"(bytes) : "memory");
}

static __device__ __forceinline__ bool
_mbar_try (uint64_t *bar, uint32_t parity)
{
  uint32_t ok;

  asm volatile ("{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.b32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(_smem_u32 (bar)), "r"(parity)
                : "memory");

  return ok != 0;
}

static __device__ __forceinline__ uint64_t
_globaltimer (void)
{
  uint64_t t;

  asm volatile ("mov.u64 %0, %%globaltimer;" : "=l"(t));

  return t;
}

/* Bounded wait: gives up after TC_WAIT_NS of wall time (setting the CTA error
 * flag) and, with bail set, as soon as another role has raised the flag. */
#define TC_WAIT_NS 1500000000ull

static __device__ __forceinline__ bool
_mbar_wait (uint64_t *bar, uint32_t parity, volatile int *err, bool bail = true)
{
  if (_mbar_try (bar, parity))
    return true;

  const uint64_t t0 = _globaltimer ();

  for (uint32_t i = 1;; i++)
  {
    if (_mbar_try (bar, parity))
      return true;

    if ((i & 63u) == 0u)
    {
      if (bail && *err)
        return false;

      if (_globaltimer () - t0 > TC_WAIT_NS)
        break;
    }
  }

  *err = 1;

  return false;
}

static __device__ __forceinline__ void
_bulk_g2s (void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
  asm volatile ("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(_smem_u32 (dst)), "l"(src), "r"(bytes), "r"(_smem_u32 (bar))
                : "memory");
}

/* shared-memory matrix descriptor: K-major, no swizzle, version 1 (bit 46) */
static __device__ __forceinline__ uint64_t
_sdesc (const void *p, uint32_t lbo)
{
  const uint64_t a = (uint64_t) _smem_u32 (p);

  return ((a & 0x3FFFFull) >> 4) | ((uint64_t) (lbo >> 4) << 16) | ((uint64_t) (TC_SBO >> 4) << 32) | (1ull << 46);
}

static __device__ __forceinline__ void
_mma_commit (uint64_t *bar)
{
  asm volatile ("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                ::"r"(_smem_u32 (bar))
                : "memory");
}

static __device__ __forceinline__ void
_tc_fence_before (void)
{
  asm volatile ("tcgen05.fence::before_thread_sync;" ::: "memory");
}

static __device__ __forceinline__ void
_tc_fence_after (void)
{
  asm volatile ("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* two 32-column TMEM loads in flight and their wait in one asm statement, so
 * no register the loads write is touched before the wait */
static __device__ __forceinline__ void
_tmem_ld64 (uint32_t t0, uint32_t t1, float *v)
{
  uint32_t r[64];

  asm volatile ("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
                "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
                "tcgen05.wait::ld.sync.aligned;"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]),
                  "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
                  "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]),
                  "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
                  "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
                : "r"(t0), "r"(t1)
                : "memory");

#pragma unroll
  for (int i = 0; i < 64; i++)
    v[i] = __uint_as_float (r[i]);
}

static __device__ __forceinline__ float
_tf32 (float x)
{
  uint32_t r;

  asm ("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));

  return __uint_as_float (r);
}

/* byte offset of element (row, k) in a chunk-outer K-major tile with lbo = R/8*128 */
static __device__ __forceinline__ uint32_t
_cm_off (int row, int k, uint32_t lbo)
{
  return (uint32_t) ((k >> 2) * lbo + (row >> 3) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

#endif /* NCG_TC_PTX_CUH */
