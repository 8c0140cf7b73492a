// Plane kernel with the x exchange through an L2-resident scratch.
//
// A group of G = Xs/R CTAs owns one (half-)plane of Xs x Y modes at a time
// (persistent, planes strided by the group count).  The group is a
// thread-block cluster (R = 16 rows per CTA), or G consecutive CTAs of a
// cooperative launch that meet at counter barriers in global memory (a 16-CTA
// cluster must fit in one GPC, which leaves a quarter of the SMs idle); from
// 256-wide planes a cooperative launch of the diffraction kernel uses R = 8
// rows per 4-warp CTA, twice the CTAs per SM:
//   1. each CTA loads R rows (cp.async, prefetched during the previous
//      plane), runs the forward y FFT in shared memory and writes the rows to
//      the group's scratch buffer in global memory (it stays in L2);
//   2. group barrier; each CTA takes Yc = Y/G y-columns of all Xs rows from
//      the scratch, runs the forward x FFT, the per-mode multiplier and the
//      inverse x FFT (the middle four-step stage, multiplier and its inverse
//      never leave registers), and writes the columns back;
//   3. group barrier; each CTA reads its rows back, runs the inverse y FFT
//      and stores the rows to HBM.
// One scratch half-plane per group suffices with two barriers per plane:
// stages 1 and 3 of a CTA touch only its own rows (the split-phase flow uses
// two).  Shared memory holds either R rows or Xs x Yc columns: about 64 KB
// with 16 rows for 512 x 512 planes split in halves (two CTAs per SM), 32 KB
// with 8 rows (four CTAs per SM).
//
// Reference semantics are those of the plane kernels in asg_xykernel.cu
// (angular_spectrum_solver.py :649-655, :667-685, :630-643).
#include <cooperative_groups.h>

#include "asg_internal.h"

namespace cg = cooperative_groups;

ASG_DEFINE_ROOT_UPLOADER(asg_roots_upload_l2)

namespace {

ASG_DEV void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
ASG_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
ASG_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

ASG_DEV bool is_dc_or_nyq_l2(int f, int nT) { return f == 0 || 2 * f == nT; }

// ---- bulk (TMA) row loads --------------------------------------------------
// The spectrum rows a warp transforms in stage 1 come from HBM as 1-D bulk
// async copies (cp.async.bulk, the copy engine moves them; one instruction per
// segment instead of one 16-byte cp.async per lane), one segment per N2 slots
// (the padded row layout puts two slots of padding after every N2), completing
// on the warp's own mbarrier.  Segments are N2 * 8 bytes (128, 192 or 256),
// row strides and segment offsets in shared memory multiples of 16 bytes, and
// the sources are rows of a cudaMalloc'd spectrum: every bulk-copy alignment
// rule holds for the supported planes (Y in 128..512).  The rows were written
// by an earlier kernel, so no proxy fence is needed on the global side.
ASG_DEV unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
ASG_DEV void mbar_init(uint64_t* mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count) : "memory");
}
ASG_DEV void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
ASG_DEV void mbar_expect_tx(uint64_t* mb, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)),
               "r"(bytes) : "memory");
}
ASG_DEV bool mbar_try_wait(uint64_t* mb, unsigned parity) {
  unsigned ok = 0;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok) : "r"(smem_u32(mb)), "r"(parity) : "memory");
  return ok != 0;
}
ASG_DEV void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* mb) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(mb)) : "memory");
}
// orders this thread's earlier generic accesses to shared memory before later
// async-proxy (bulk copy) writes to it
ASG_DEV void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// A warp's bulk loads of RPW rows: every lane fences its generic accesses to
// the rows, lane 0 arms the mbarrier with the byte count, the lanes issue the
// segments.  rows_src(j) gives the global start of row j, rows_dst(j) its
// shared-memory row.
template <class PY, int RPW, class Src, class Dst>
ASG_DEV void warp_bulk_rows(uint64_t* mb, int lane, Src rows_src, Dst rows_dst) {
  constexpr int SEG = PY::N2;              // slots per segment
  constexpr int NSEG = PY::N / SEG;         // segments per row
  constexpr unsigned BYTES = SEG * sizeof(float2);
  static_assert(BYTES % 16 == 0 && ((SEG + 2) * sizeof(float2)) % 16 == 0 &&
                    (PY::PADDED * sizeof(float2)) % 16 == 0,
                "bulk-copy alignment");
  fence_proxy_async_smem();
  __syncwarp();
  if (lane == 0) mbar_expect_tx(mb, RPW * NSEG * BYTES);
  __syncwarp();
  for (int i = lane; i < RPW * NSEG; i += 32) {
    const int j = i / NSEG, sg = i - j * NSEG;
    bulk_g2s(rows_dst(j) + sg * (SEG + 2), rows_src(j) + sg * SEG, BYTES, mb);
  }
}

// Bounded wait for the warp's mbarrier phase `parity`: gives up after one
// second (or as soon as the status word is set), records ASG_ERR_TIMEOUT if
// nothing else was recorded, and returns false.
ASG_DEV bool mbar_wait_bounded(uint64_t* mb, unsigned parity, unsigned* status) {
  unsigned long long t0 = 0;
  for (unsigned it = 0;; ++it) {
    if (mbar_try_wait(mb, parity)) return true;
    if ((it & 63) == 63) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > 1000000000ull) {
        atomicCAS(status, 0u, (unsigned)(-ASG_ERR_TIMEOUT));
        return false;
      }
    }
  }
}

ASG_DEV bool l2_should_skip(const XYParams& p) {
  if (*((volatile const unsigned*)p.status) != 0u) return true;
  if (p.check_stability) {
    const float m = __uint_as_float(*p.max_cur);
    const bool nan = (m != m) || isinf(m);
    const bool bad = nan || (p.stab_coef * (double)m > p.stab_thr);
    if (bad) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (atomicCAS(p.status, 0u, (unsigned)(nan ? -ASG_ERR_NAN : -ASG_ERR_STABILITY)) == 0u)
          *p.status_step = *p.step;
      }
      return true;
    }
  }
  return false;
}

ASG_DEV unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier of the G CTAs of one group when the kernel runs as a cooperative
// launch (every CTA of the grid is resident) instead of thread-block
// clusters: CTA arrivals are counted in global memory, with fences on both
// sides so that the group's scratch writes before the barrier are visible to
// its reads after it (the reads go to L2: cp.async.cg).  `target` is G times
// the number of barriers passed so far.  The wait gives up after one second,
// or as soon as the status word is set, records ASG_ERR_TIMEOUT (if nothing
// else was recorded) and returns false; the caller then leaves the kernel.
ASG_DEV bool group_barrier(unsigned* cnt, unsigned target, unsigned* status, int* ok_s) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(cnt, 1u);
    const unsigned long long t0 = global_ns();
    while (*((volatile unsigned*)cnt) < target) {
      if (*((volatile unsigned*)status) != 0u) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > 1000000000ull) {
        atomicCAS(status, 0u, (unsigned)(-ASG_ERR_TIMEOUT));
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    *ok_s = ok;
  }
  __syncthreads();
  return *ok_s != 0;
}

}  // namespace

// Blocks per SM.  With 8-warp blocks, planes up to 384 wide run three per SM
// (80 registers without spills; the diffraction kernel then reads its twiddle
// and class tables through L1 to keep its shared memory to the row buffer; the
// closing kernel fits as it is): 4-7 % faster than two.  512-wide planes keep
// two, the diffraction kernel's tables in shared memory (at 80 registers their
// 32-point row transform spills, and the closing kernel's shared memory allows
// two).  The diffraction kernel's 4-warp blocks of a cooperative launch (8
// rows per CTA) run twice as many blocks per SM with the same registers.
template <class PY, int NT>
struct L2Shape {
  static constexpr bool kTablesInSmem = PY::N >= 512;
  static constexpr int kMinBlocks = (kTablesInSmem ? 2 : 3) * (NT == 128 ? 2 : 1);
};

template <class PY, class PX, int R, int NT>
__global__ void __launch_bounds__(NT, L2Shape<PY, NT>::kMinBlocks) xy_l2(XYParams p) {
  constexpr int Y = PY::N, RS = PY::PADDED;
  constexpr int Xs = PX::N;
  constexpr int NW = NT / 32;
  constexpr int G = Xs / R;          // CTAs per cluster (the launcher checks p.G == G)
  constexpr int Yc = Y / G;          // y-columns per CTA in stage 2
  constexpr int TS = Yc;             // row stride of the column tile (complex): lanes run
                                     // along c, so the strided x accesses are conflict free
  static_assert(Xs % R == 0 && Y % G == 0 && Yc % 2 == 0, "tile shape");
  constexpr int RPW = R / NW;        // rows per warp in stages 1 and 3
  static_assert(R % NW == 0, "rows per warp");
  extern __shared__ float4 smraw[];
  float2* buf = reinterpret_cast<float2*>(smraw);       // rows [R][RS] or tile [Xs][TS]
  __shared__ float red[2][NW];

  constexpr bool TS_SMEM = L2Shape<PY, NT>::kTablesInSmem;
  const int nbuf = p.l2_buf_elems;   // max(R*RS, Xs*TS), set by the host
  float2* tw_y_s = buf + nbuf;
  float2* tw_x_s = tw_y_s + Y;
  int* clsy_s = reinterpret_cast<int*>(tw_x_s + Xs);
  int* clsx_s = clsy_s + Y;           // [nsub][Xs] by x slot of the Xs-point FFT
  const float2* tw_y = TS_SMEM ? tw_y_s : p.twY;
  const int* clsy = TS_SMEM ? clsy_s : p.cls_y;
  const int* clsx = TS_SMEM ? clsx_s : p.l2_cls_x;

  cg::cluster_group cl = cg::this_cluster();
  const bool coop = p.coop != 0;
  const int rank = coop ? (int)(blockIdx.x % G) : (G > 1) ? (int)cl.block_rank() : 0;
  const int cid = blockIdx.x / G, ncl = gridDim.x / G;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int sync_ok;
  __shared__ uint64_t row_mbar[NW];  // bulk row loads of each warp
  __shared__ int rows_failed;
  unsigned arrivals = 0;
  // the group barrier: cluster barrier, or the counter barrier of a cooperative launch
  auto gsync = [&]() -> bool {
    if (coop) {
      arrivals += G;
      return group_barrier(p.grp_cnt + cid, arrivals + p.grp_skew, p.status, &sync_ok);
    }
    if (G > 1) cl.sync();
    else __syncthreads();
    return true;
  };
  const int nsub = p.nsub;
  const int nq = p.nplanes * nsub;
  if (l2_should_skip(p)) return;
  if (lane == 0) {
    mbar_init(&row_mbar[warp], 1);
    mbar_init_fence();
  }
  if (tid == 0) rows_failed = 0;
  __syncthreads();
  unsigned row_phase = 0;
  bool row_pending = false;

  if constexpr (TS_SMEM) {
    for (int i = tid; i < Y; i += NT) {
      tw_y_s[i] = p.twY[i];
      clsy_s[i] = p.cls_y[i];
    }
    for (int i = tid; i < Xs; i += NT) tw_x_s[i] = p.twX[i * nsub];  // W_Xs^i
    for (int i = tid; i < nsub * Xs; i += NT) clsx_s[i] = p.l2_cls_x[i];
  }
  const int nsub_l = nsub;
  auto tw_x = [&](int i) { return TS_SMEM ? tw_x_s[i] : __ldg(p.twX + i * nsub_l); };
  float2* scratch0 = p.l2_scratch + (size_t)cid * 2 * Xs * Y;

  auto zero_plane = [&](int q) {
    return p.zero_dc_nyq && is_dc_or_nyq_l2(p.f_of_plane[q / nsub], p.nT);
  };
  auto sub_base = [&](int q) {
    const int plane = q / nsub, h = q - (q / nsub) * nsub;
    return p.spec + ((size_t)plane * p.X + (size_t)h * Xs) * Y;
  };
  // loads of my warp's rows of (sub-)plane q: bulk copies, or 16-byte cp.async
  const bool bulk = p.bulk_rows != 0;
  auto load_rows = [&](int q) {
    const float2* g0 = sub_base(q) + (size_t)(rank * R + warp) * Y;
    float2* d0 = buf + warp * RS;
    if (bulk) {
      warp_bulk_rows<PY, RPW>(
          &row_mbar[warp], lane, [&](int j) { return g0 + (size_t)NW * j * Y; },
          [&](int j) { return d0 + NW * j * RS; });
      row_pending = true;
    } else {
#pragma unroll
      for (int j = 0; j < RPW; ++j)
        for (int s2 = lane; s2 < Y / 2; s2 += 32)
          cp_async16(d0 + NW * j * RS + PY::pos(2 * s2), g0 + (size_t)NW * j * Y + 2 * s2);
      cp_async_commit();
    }
  };
  // waits for my warp's rows, then for the whole block; false after a timeout
  auto wait_rows = [&]() -> bool {
    if (row_pending) {
      if (!mbar_wait_bounded(&row_mbar[warp], row_phase, p.status)) rows_failed = 1;
      row_phase ^= 1u;
      row_pending = false;
    }
    cp_async_wait_all();
    __syncthreads();
    return rows_failed == 0;
  };
  auto zero_rows = [&](int q) {
    float4* g4 = reinterpret_cast<float4*>(sub_base(q) + (size_t)rank * R * Y);
    for (int i = tid; i < R * Y / 2; i += NT) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  };

  // ---- 1. forward y FFT on my rows (warp w: rows w + NW j, both rows'
  //      tasks share the warp's lanes), rows -> scratch S (slot order) ----
  auto stage1 = [&](float2* S) {
    for (int i = lane; i < RPW * PY::N2; i += 32) {
      const int j = i / PY::N2, b = i - j * PY::N2;
      stepA_fwd_smem<PY, false>(buf + (warp + NW * j) * RS, b, tw_y);
    }
    __syncwarp();
    for (int i = lane; i < RPW * PY::N1; i += 32) {
      const int j = i / PY::N1, ka = i - j * PY::N1;
      stepB_smem<PY, false>(buf + (warp + NW * j) * RS, ka);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < RPW; ++j) {
      const int r = warp + NW * j;
      const float2* row = buf + r * RS;
      float4* dst = reinterpret_cast<float4*>(S + (size_t)(rank * R + r) * Y);
      for (int s2 = lane; s2 < Y / 2; s2 += 32)
        dst[s2] = *reinterpret_cast<const float4*>(row + PY::pos(2 * s2));
    }
  };

  // ---- 2. columns [rank*Yc, +Yc) of all Xs rows: x FFT, multiplier (or the
  //      power sums), inverse; ends with the block's tile writes to S issued ----
  auto stage2 = [&](int q, float2* S) {
    const int plane = q / nsub, h = q - (q / nsub) * nsub;
    const int c0 = rank * Yc;
    // tile[x][c], row stride TS
    for (int i = tid; i < Xs * Yc / 2; i += NT) {
      const int x = i / (Yc / 2), c2 = 2 * (i - x * (Yc / 2));
      cp_async16(buf + x * TS + c2, S + (size_t)x * Y + c0 + c2);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    // step A (forward): task (b, c), elements x = b + N2x*a
    for (int it = tid; it < PX::N2 * Yc; it += NT) {
      const int b = it / Yc, c = it - b * Yc;
      float2 v[PX::N1];
#pragma unroll
      for (int a = 0; a < PX::N1; ++a) v[a] = buf[(b + PX::N2 * a) * TS + c];
      dft<PX::N1, false>(v);
      buf[b * TS + c] = v[0];
#pragma unroll
      for (int ka = 1; ka < PX::N1; ++ka) buf[(b + PX::N2 * ka) * TS + c] = cmul(v[ka], tw_x(b * ka));
    }
    __syncthreads();
    float psum = 0.f, pden = 0.f;
    // step B forward, multiplier, step B inverse: task (ka, c), slots kb + N2x*ka
    for (int it = tid; it < PX::N1 * Yc; it += NT) {
      const int ka = it / Yc, c = it - ka * Yc;
      float2 v[PX::N2];
#pragma unroll
      for (int b = 0; b < PX::N2; ++b) v[b] = buf[(b + PX::N2 * ka) * TS + c];
      dft<PX::N2, false>(v);
      const int cy = clsy[c0 + c];
      const int* cxh = clsx + h * Xs;
      if (p.power_only) {
        const float* ot = p.obl_table + (size_t)plane * p.ncx * p.ncy + cy;
#pragma unroll
        for (int kb = 0; kb < PX::N2; ++kb) {
          const float o = ot[cxh[kb + PX::N2 * ka]];
          const float P = v[kb].x * v[kb].x + v[kb].y * v[kb].y;
          psum = fmaf(P, o, psum);
          pden += (o > 0.f) ? P : 0.f;
        }
        continue;
      }
      if (p.table != nullptr) {
        const float2* tt = p.table + (size_t)plane * p.ncx * p.ncy + cy;
#pragma unroll
        for (int kb = 0; kb < PX::N2; ++kb)
          v[kb] = cmul(v[kb], tt[cxh[kb + PX::N2 * ka]]);
      } else {
        const float nrm = 1.0f / ((float)Xs * (float)Y);
#pragma unroll
        for (int kb = 0; kb < PX::N2; ++kb) v[kb] = cscale(v[kb], nrm);
      }
      dft<PX::N2, true>(v);
#pragma unroll
      for (int b = 0; b < PX::N2; ++b) buf[(b + PX::N2 * ka) * TS + c] = v[b];
    }
    if (p.power_only) {
      psum = warp_sum(psum);
      pden = warp_sum(pden);
      if (lane == 0) {
        red[0][warp] = psum;
        red[1][warp] = pden;
      }
      __syncthreads();
      if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < NW; ++w) {
          a += (double)red[0][w];
          b += (double)red[1][w];
        }
        atomicAdd(p.power_acc, a);
        atomicAdd(p.power_acc + 1, b);
      }
      return;
    }
    __syncthreads();
    // step A inverse: task (b, c)
    for (int it = tid; it < PX::N2 * Yc; it += NT) {
      const int b = it / Yc, c = it - b * Yc;
      float2 v[PX::N1];
      v[0] = buf[b * TS + c];
#pragma unroll
      for (int ka = 1; ka < PX::N1; ++ka) v[ka] = cmulc(buf[(b + PX::N2 * ka) * TS + c], tw_x(b * ka));
      dft<PX::N1, true>(v);
#pragma unroll
      for (int a = 0; a < PX::N1; ++a) buf[(b + PX::N2 * a) * TS + c] = v[a];
    }
    __syncthreads();
    for (int i = tid; i < Xs * Yc / 2; i += NT) {
      const int x = i / (Yc / 2), c2 = 2 * (i - x * (Yc / 2));
      *reinterpret_cast<float4*>(S + (size_t)x * Y + c0 + c2) =
          *reinterpret_cast<const float4*>(buf + x * TS + c2);
    }
  };

  // ---- 3. my rows back from the scratch (cp.async.cg reads L2: other CTAs
  //      wrote these rows; each warp copies and then transforms only its own
  //      rows), inverse y FFT, store ----
  auto stage3 = [&](int q, float2* S) {
#pragma unroll
    for (int j = 0; j < RPW; ++j) {
      const int r = warp + NW * j;
      const float2* srcr = S + (size_t)(rank * R + r) * Y;
      float2* row = buf + r * RS;
      for (int s2 = lane; s2 < Y / 2; s2 += 32) cp_async16(row + PY::pos(2 * s2), srcr + 2 * s2);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
    float2* gbase = sub_base(q) + (size_t)rank * R * Y;
    for (int i = lane; i < RPW * PY::N1; i += 32) {
      const int j = i / PY::N1, ka = i - j * PY::N1;
      stepB_smem<PY, true>(buf + (warp + NW * j) * RS, ka);
    }
    __syncwarp();
    for (int i = lane; i < RPW * PY::N2; i += 32) {
      const int j = i / PY::N2, b = i - j * PY::N2;
      const int r = warp + NW * j;
      const float2* row = buf + r * RS;
      float2* grow = gbase + (size_t)r * Y;
      float2 v[PY::N1];
      v[0] = row[PY::pos(b)];
#pragma unroll
      for (int ka = 1; ka < PY::N1; ++ka) v[ka] = cmulc(row[PY::pos(b + PY::N2 * ka)], tw_y[b * ka]);
      dft<PY::N1, true>(v);
#pragma unroll
      for (int a = 0; a < PY::N1; ++a) grow[b + PY::N2 * a] = v[a];
    }
    __syncwarp();
  };
  auto next_plane = [&](int q) {
    q += ncl;
    while (q < nq && zero_plane(q)) q += ncl;
    return q;
  };

  if (coop && p.pipe && !p.power_only) {
    // ---- pipelined flow: split-phase counter barriers over two scratch halves.
    // Per plane i: arrive at barrier 1 after stage 1, wait before stage 2;
    // arrive at barrier 2 after stage 2, wait before stage 3.  Between the
    // arrival at barrier 2 of plane i and its wait, the block runs stage 1 of
    // plane i+1 (into the other scratch half); between the arrival at barrier
    // 1 of plane i+1 and its wait, stage 3 of plane i.  Two counters per group
    // (arrivals at the two barriers) with targets G (i + 1): arriving at a
    // barrier for plane i+1 needs the wait of plane i at the same barrier,
    // so a count can only reach its target through the arrivals it waits for.
    // Scratch half i&1: stage 1 of plane i+2 rewrites my rows of it only after
    // my stage 3 of plane i (program order), and every block's stage 2 of
    // plane i+2 only after barrier 1 of plane i+2, which every block reaches
    // after its own stage 3 of plane i.
    unsigned* c1 = p.grp_cnt + cid;
    unsigned* c2 = p.grp_cnt + p.l2_max_clusters + cid;
    auto arrive = [&](unsigned* cnt) {
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        atomicAdd(cnt, 1u);
      }
    };
    auto wait = [&](unsigned* cnt, unsigned target) -> bool {
      if (tid == 0) {
        int ok = 1;
        const unsigned long long t0 = global_ns();
        while (*((volatile unsigned*)cnt) < target) {
          if (*((volatile unsigned*)p.status) != 0u) {
            ok = 0;
            break;
          }
          if (global_ns() - t0 > 1000000000ull) {
            atomicCAS(p.status, 0u, (unsigned)(-ASG_ERR_TIMEOUT));
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
        __threadfence();
        sync_ok = ok;
      }
      __syncthreads();
      return sync_ok != 0;
    };
    for (int q = cid; q < nq; q += ncl)
      if (zero_plane(q)) zero_rows(q);
    int q = cid;
    while (q < nq && zero_plane(q)) q += ncl;
    if (q < nq) {
      load_rows(q);
      if (wait_rows()) {
        stage1(scratch0);
        arrive(c1);
      } else {
        q = nq;
      }
    }
    for (unsigned i = 0; q < nq; ++i) {
      float2* Sc = scratch0 + (size_t)(i & 1u) * Xs * Y;
      float2* Sn = scratch0 + (size_t)((i + 1) & 1u) * Xs * Y;
      if (!wait(c1, G * (i + 1) + p.grp_skew)) break;
      stage2(q, Sc);
      const int qn = next_plane(q);
      __syncthreads();  // the tile is written out: the row buffer is free
      if (qn < nq) load_rows(qn);
      arrive(c2);
      if (qn < nq) {
        if (!wait_rows()) break;
        stage1(Sn);
        arrive(c1);
      }
      if (!wait(c2, G * (i + 1) + p.grp_skew)) break;
      stage3(q, Sc);
      q = qn;
    }
  } else {
    int issued = -1;
    for (int q = cid; q < nq; q += ncl) {
      if (zero_plane(q)) {
        zero_rows(q);
        continue;
      }
      // one scratch half-plane per cluster: in stages 1 and 3 each CTA touches
      // only its own rows, and the cluster barriers order stage 2's accesses to
      // all rows after every CTA's stage 3 of the previous plane
      float2* S = scratch0;
      if (issued != q) load_rows(q);
      if (!wait_rows()) break;
      stage1(S);
      // the barrier (release / acquire) orders these global writes before the
      // other CTAs' reads of the scratch
      if (!gsync()) break;
      stage2(q, S);
      // power sums: no CTA reuses the scratch before every CTA has read it
      if (!gsync()) break;
      if (p.power_only) continue;
      stage3(q, S);
      const int qn = next_plane(q);
      if (qn < nq) {
        load_rows(qn);
        issued = qn;
      }
    }
  }
  cp_async_wait_all();
  // no bulk copy may still be landing in shared memory when the block exits
  if (row_pending) mbar_wait_bounded(&row_mbar[warp], row_phase, p.status);
}

// ---------------------------------------------------------------------------
// Closing-stage plane kernel: the attenuation multiplier with the boundary and
// screen epilogue fused, whole planes out.
//
// One cluster owns both half-planes of a plane (the column pass applied the
// first radix-2 x stage, so rows x < X/2 hold a and rows x >= X/2 hold b):
//   1. each CTA runs the forward y FFT on its R rows of a and of b and writes
//      them to the cluster's scratch (rows of a, then rows of b);
//   2. cluster barrier; per round of YR y-columns, each CTA loads the a and b
//      tiles, runs the forward x FFT, the multiplier and the inverse x FFT of
//      both, recombines s(x) = a + W_X^-x b, s(x + X/2) = a - W_X^-x b, and
//      applies the parts of the epilogue that act along x only: the x factor
//      of the frequency-weighted damping and the Engquist-Majda x edges.  They
//      commute with the y transform (coefficients independent of y), so they
//      run here on y-spectral data with whole x columns at hand;
//   3. cluster barrier; each CTA reads its whole-plane rows, runs the inverse
//      y FFT and applies, along the row, the y factor of the damping, the
//      Engquist-Majda y edges and the phase/amplitude screens, then stores.
// The order of the epilogue is that of the reference (damping, x edges, then
// y edges on the x-corrected values, then screens): the y factor of the
// damping commutes with the x edges.  Re() of bins 0 and nT/2, which the
// reference takes between the operators, commutes with all of them on bin 0
// (real coefficients there) and is left to the column pass; the Nyquist plane
// (p.skip_plane) gets no epilogue here and goes through the epilogue pass.
// Each CTA reads and writes only its own rows in stages 1 and 3, so one
// scratch plane per cluster needs no barrier between consecutive planes.
// (angular_spectrum_solver.py :667-685, :658-664, :144-179, :185-272,
// :352-390, :1494-1518)
// ---------------------------------------------------------------------------
template <class PY, class PX, int R, int NT>
__global__ void __launch_bounds__(NT, L2Shape<PY, NT>::kMinBlocks) xy_l2c(XYParams p) {
  constexpr int Y = PY::N, RS = PY::PADDED;
  constexpr int Xs = PX::N, X = 2 * Xs;
  constexpr int NW = NT / 32;
  constexpr int G = Xs / R;
  constexpr int Yc = Y / G;                 // y-columns per CTA in stage 2
  constexpr int YR = Yc < 16 ? Yc : 16;     // columns per round: tiles [2][Xs][YR]
  constexpr int NRND = Yc / YR;
  constexpr int TS = YR;
  constexpr int RPW = R / NW;
  static_assert(Xs % R == 0 && Y % G == 0 && Yc % YR == 0 && YR % 2 == 0, "tile shape");
  static_assert(R % NW == 0 && NT % YR == 0 && X % (NT / YR) == 0, "thread layout");
  constexpr int CHUNK = X / (NT / YR);      // x per thread in the x-edge walk
  extern __shared__ float4 smraw[];
  float2* buf = reinterpret_cast<float2*>(smraw);     // rows [R][RS] or tiles [2][Xs][TS]
  const int nbuf = p.l2_buf_elems;
  float2* tw_y = buf + nbuf;
  float2* tw_x = tw_y + Y;
  float* gxs = reinterpret_cast<float*>(tw_x + Xs);   // [X] damping x factor, this plane
  float* gys = gxs + X;                               // [Y] damping y factor, this plane
  float* wxs = gys + Y;                               // [X] Engquist-Majda weights
  float* wys = wxs + X;                               // [Y]
  int* clsy = reinterpret_cast<int*>(wys + Y);
  int* clsx = clsy + Y;                               // [2][Xs]

  cg::cluster_group cl = cg::this_cluster();
  const bool coop = p.coop != 0;
  const int rank = coop ? (int)(blockIdx.x % G) : (G > 1) ? (int)cl.block_rank() : 0;
  const int cid = blockIdx.x / G, ncl = gridDim.x / G;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (*((volatile const unsigned*)p.status) != 0u) return;
  __shared__ int sync_ok;
  __shared__ uint64_t row_mbar[NW];  // bulk row loads of each warp
  if (lane == 0) {
    mbar_init(&row_mbar[warp], 1);
    mbar_init_fence();
  }
  __syncwarp();
  unsigned row_phase = 0;
  bool row_pending = false;
  unsigned arrivals = 0;
  auto gsync = [&]() -> bool {
    if (coop) {
      arrivals += G;
      return group_barrier(p.grp_cnt + cid, arrivals + p.grp_skew, p.status, &sync_ok);
    }
    if (G > 1) cl.sync();
    else __syncthreads();
    return true;
  };

  for (int i = tid; i < Y; i += NT) {
    tw_y[i] = p.twY[i];
    clsy[i] = p.cls_y[i];
    wys[i] = (p.epi & EPI_SUPERABS) ? p.sa_wy[i] : 0.f;
  }
  for (int i = tid; i < Xs; i += NT) tw_x[i] = p.twX[i * 2];  // W_Xs^i
  for (int i = tid; i < 2 * Xs; i += NT) {
    clsx[i] = p.l2_cls_x[i];
    wxs[i] = (p.epi & EPI_SUPERABS) ? p.sa_wx[i] : 0.f;
  }
  float2* S = p.l2_scratch + (size_t)cid * X * Y;     // rows of a, then rows of b
  // chunks of the x-edge walk that hold Engquist-Majda weights (fixed per launch)
  __shared__ unsigned char x_chunk_any[NT / YR];
  __syncthreads();
  if (tid < NT / YR) {
    bool any = false;
    for (int x = tid * CHUNK; x < (tid + 1) * CHUNK; ++x) any |= wxs[x] != 0.f;
    x_chunk_any[tid] = any ? 1 : 0;
  }
  const bool fw = (p.epi & EPI_FREQW) != 0, sa = (p.epi & EPI_SUPERABS) != 0;
  const float st = p.sa_strength;

  // loads of my warp's rows of half-plane h of `plane`: bulk copies (bulk_rows
  // 2), or 16-byte cp.async
  const bool bulk = p.bulk_rows >= 2;
  auto prefetch_rows = [&](int plane, int h) {
    const float2* g0 = p.spec + ((size_t)plane * X + (size_t)h * Xs + rank * R + warp) * Y;
    float2* d0 = buf + warp * RS;
    if (bulk) {
      warp_bulk_rows<PY, RPW>(
          &row_mbar[warp], lane, [&](int j) { return g0 + (size_t)NW * j * Y; },
          [&](int j) { return d0 + NW * j * RS; });
      row_pending = true;
    } else {
#pragma unroll
      for (int j = 0; j < RPW; ++j)
        for (int s2 = lane; s2 < Y / 2; s2 += 32)
          cp_async16(d0 + NW * j * RS + PY::pos(2 * s2), g0 + (size_t)NW * j * Y + 2 * s2);
      cp_async_commit();
    }
  };
  int issued = -1;

  for (int plane = cid; plane < p.nplanes; plane += ncl) {
    const bool epi = plane != p.skip_plane && (p.epi != 0 || p.nscreens > 0);
    const float cf = sa ? p.sa_coef[plane] : 0.f;   // coeff = -i cf
    __syncthreads();  // previous plane's users of gxs/gys are done
    if (fw && epi) {
      const float e = p.fw_exp[plane];
      for (int i = tid; i < X; i += NT) gxs[i] = exp2f(e * p.fw_lx[i]);
      for (int i = tid; i < Y; i += NT) gys[i] = exp2f(e * p.fw_ly[i]);
    }
    // ---- 1. forward y FFT of my rows of a and of b -> scratch; each warp
    //      loads, transforms and stores only its own rows, so it issues the
    //      loads of its rows of b as soon as its rows of a are stored ----
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      if (issued != plane * 2 + h) prefetch_rows(plane, h);
      if (row_pending) {
        // on a timeout the status word is set and the run ends with it
        mbar_wait_bounded(&row_mbar[warp], row_phase, p.status);
        row_phase ^= 1u;
        row_pending = false;
      }
      cp_async_wait_all();
      __syncwarp();
      for (int i = lane; i < RPW * PY::N2; i += 32) {
        const int j = i / PY::N2, b = i - j * PY::N2;
        stepA_fwd_smem<PY, false>(buf + (warp + NW * j) * RS, b, tw_y);
      }
      __syncwarp();
      for (int i = lane; i < RPW * PY::N1; i += 32) {
        const int j = i / PY::N1, ka = i - j * PY::N1;
        stepB_smem<PY, false>(buf + (warp + NW * j) * RS, ka);
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < RPW; ++j) {
        const int r = warp + NW * j;
        const float2* row = buf + r * RS;
        float4* dst = reinterpret_cast<float4*>(S + (size_t)(h * Xs + rank * R + r) * Y);
        for (int s2 = lane; s2 < Y / 2; s2 += 32)
          dst[s2] = *reinterpret_cast<const float4*>(row + PY::pos(2 * s2));
      }
      __syncwarp();  // my rows are reloaded next
    }
    if (!gsync()) break;

    // ---- 2. per round: x FFT, multiplier, inverse, recombination, x edges ----
#pragma unroll 1
    for (int rnd = 0; rnd < NRND; ++rnd) {
      const int c0 = rank * Yc + rnd * YR;
      float2* tile = buf;  // [h][x][c], h-stride Xs*TS
      for (int i = tid; i < 2 * Xs * YR / 2; i += NT) {
        const int hx = i / (YR / 2), c2 = 2 * (i - hx * (YR / 2));
        cp_async16(tile + hx * TS + c2, S + (size_t)hx * Y + c0 + c2);
      }
      cp_async_commit();
      cp_async_wait_all();
      __syncthreads();
      for (int it = tid; it < 2 * PX::N2 * YR; it += NT) {
        const int hb = it / YR, c = it - hb * YR;
        const int h = hb / PX::N2, b = hb - h * PX::N2;
        float2* t = tile + h * Xs * TS;
        float2 v[PX::N1];
#pragma unroll
        for (int a = 0; a < PX::N1; ++a) v[a] = t[(b + PX::N2 * a) * TS + c];
        dft<PX::N1, false>(v);
        t[b * TS + c] = v[0];
#pragma unroll
        for (int ka = 1; ka < PX::N1; ++ka) t[(b + PX::N2 * ka) * TS + c] = cmul(v[ka], tw_x[b * ka]);
      }
      __syncthreads();
      for (int it = tid; it < 2 * PX::N1 * YR; it += NT) {
        const int hk = it / YR, c = it - hk * YR;
        const int h = hk / PX::N1, ka = hk - h * PX::N1;
        float2* t = tile + h * Xs * TS;
        float2 v[PX::N2];
#pragma unroll
        for (int b = 0; b < PX::N2; ++b) v[b] = t[(b + PX::N2 * ka) * TS + c];
        dft<PX::N2, false>(v);
        const int* cxh = clsx + h * Xs;
        if (p.table != nullptr) {
          const float2* tt = p.table + (size_t)plane * p.ncx * p.ncy + clsy[c0 + c];
#pragma unroll
          for (int kb = 0; kb < PX::N2; ++kb)
            v[kb] = cmul(v[kb], tt[cxh[kb + PX::N2 * ka]]);
        } else {
          const float nrm = 1.0f / ((float)Xs * (float)Y);
#pragma unroll
          for (int kb = 0; kb < PX::N2; ++kb) v[kb] = cscale(v[kb], nrm);
        }
        dft<PX::N2, true>(v);
#pragma unroll
        for (int b = 0; b < PX::N2; ++b) t[(b + PX::N2 * ka) * TS + c] = v[b];
      }
      __syncthreads();
      // inverse step A of both halves for task (b, c), then on the task's own
      // x = b + N2x*a, in registers, the recombination s(x) = a + W_X^-x b,
      // s(x + Xs) = a - W_X^-x b (+ damping x factor): tile h=0 <- s(x),
      // h=1 <- s(x + Xs)
      for (int it = tid; it < PX::N2 * YR; it += NT) {
        const int b = it / YR, c = it - b * YR;
        float2* ta = tile;
        float2* tb = tile + Xs * TS;
        float2 va[PX::N1], vb[PX::N1];
        va[0] = ta[b * TS + c];
        vb[0] = tb[b * TS + c];
#pragma unroll
        for (int ka = 1; ka < PX::N1; ++ka) {
          va[ka] = cmulc(ta[(b + PX::N2 * ka) * TS + c], tw_x[b * ka]);
          vb[ka] = cmulc(tb[(b + PX::N2 * ka) * TS + c], tw_x[b * ka]);
        }
        dft<PX::N1, true>(va);
        dft<PX::N1, true>(vb);
#pragma unroll
        for (int a = 0; a < PX::N1; ++a) {
          const int x = b + PX::N2 * a;
          const float2 wb = cmulc(vb[a], __ldg(p.twX + x));
          float2 s0 = cadd(va[a], wb), s1 = csub(va[a], wb);
          if (fw && epi) {
            s0 = cscale(s0, gxs[x]);
            s1 = cscale(s1, gxs[x + Xs]);
          }
          ta[x * TS + c] = s0;
          tb[x * TS + c] = s1;
        }
      }
      __syncthreads();
      if (sa && epi) {
        // x edges: thread (c, chunk) walks x0 .. x0+CHUNK-1 of column c in place,
        // with the originals of its two neighbours read before anyone writes
        const int c = tid % YR, x0 = (tid / YR) * CHUNK;
        const float2 lo = x0 > 0 ? tile[(x0 - 1) * TS + c] : make_float2(0.f, 0.f);
        const float2 hi = x0 + CHUNK < X ? tile[(x0 + CHUNK) * TS + c] : make_float2(0.f, 0.f);
        __syncthreads();
        if (x_chunk_any[tid / YR]) {
          float2 prev = lo, cur = tile[x0 * TS + c];
#pragma unroll 8
          for (int x = x0; x < x0 + CHUNK; ++x) {
            const float2 next = x + 1 < x0 + CHUNK ? tile[(x + 1) * TS + c] : hi;
            const float w = wxs[x];
            if (w != 0.f) {
              float2 d;
              if (x == 0) d = cscale(csub(next, cur), p.sa_invdx);
              else if (x == X - 1) d = cscale(csub(cur, prev), p.sa_invdx);
              else d = cscale(csub(next, prev), p.sa_inv2dx);
              const float2 cd = make_float2(cf * d.y, -cf * d.x);
              const float2 P = (x < X / 2) ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                           : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
              tile[x * TS + c] = make_float2(cur.x - st * w * P.x, cur.y - st * w * P.y);
            }
            prev = cur;
            cur = next;
          }
        }
        __syncthreads();
      }
      for (int i = tid; i < 2 * Xs * YR / 2; i += NT) {
        const int hx = i / (YR / 2), c2 = 2 * (i - hx * (YR / 2));
        *reinterpret_cast<float4*>(S + (size_t)hx * Y + c0 + c2) =
            *reinterpret_cast<const float4*>(tile + hx * TS + c2);
      }
      __syncthreads();  // tile reused by the next round
    }
    if (!gsync()) break;

    // ---- 3. my whole-plane rows: inverse y FFT, y edges, screens, store ----
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
#pragma unroll
      for (int j = 0; j < RPW; ++j) {
        const int r = warp + NW * j;
        const float2* srcr = S + (size_t)(h * Xs + rank * R + r) * Y;
        float2* row = buf + r * RS;
        for (int s2 = lane; s2 < Y / 2; s2 += 32)  // cp.async.cg reads L2: other CTAs wrote these
          cp_async16(row + PY::pos(2 * s2), srcr + 2 * s2);
      }
      cp_async_commit();
      cp_async_wait_all();
      __syncwarp();
      for (int i = lane; i < RPW * PY::N1; i += 32) {
        const int j = i / PY::N1, ka = i - j * PY::N1;
        stepB_smem<PY, true>(buf + (warp + NW * j) * RS, ka);
      }
      __syncwarp();
      // the epilogue of 32 consecutive outputs y = y0 + lane of row x: damping
      // y factor, Engquist-Majda y edges (neighbours by shuffles; lane 31's
      // right neighbour `nxt` is the undamped value at y0 + 32, lane 0's left
      // one the damped value at y0 - 1 carried in prev_last), screens, store
      auto epilogue32 = [&](int x, int y0, float2 cur, float2 nxt, float2& prev_last,
                            float2* grow) {
        const int y = y0 + lane;
        if (fw) cur = cscale(cur, gys[y]);
        float2 res = cur;
        if (sa) {
          float2 left, right;
          left.x = __shfl_up_sync(0xffffffffu, cur.x, 1);
          left.y = __shfl_up_sync(0xffffffffu, cur.y, 1);
          right.x = __shfl_down_sync(0xffffffffu, cur.x, 1);
          right.y = __shfl_down_sync(0xffffffffu, cur.y, 1);
          if (lane == 0) left = prev_last;
          if (lane == 31 && y + 1 < Y) right = fw ? cscale(nxt, gys[y + 1]) : nxt;
          const float w = wys[y];
          if (w != 0.f) {
            float2 d;
            if (y == 0) d = cscale(csub(right, cur), p.sa_invdy);
            else if (y == Y - 1) d = cscale(csub(cur, left), p.sa_invdy);
            else d = cscale(csub(right, left), p.sa_inv2dy);
            const float2 cd = make_float2(cf * d.y, -cf * d.x);
            const float2 P = (y < Y / 2) ? make_float2(0.5f * (cur.x + cd.x), 0.5f * (cur.y + cd.y))
                                         : make_float2(0.5f * (cur.x - cd.x), 0.5f * (cur.y - cd.y));
            res = make_float2(cur.x - st * w * P.x, cur.y - st * w * P.y);
          }
          prev_last.x = __shfl_sync(0xffffffffu, cur.x, 31);
          prev_last.y = __shfl_sync(0xffffffffu, cur.y, 31);
        }
        for (int k = 0; k < p.nscreens; ++k) {
          const float fs = p.screen_fscale[plane];
          const ScreenDev sc = p.screens[k];
          const size_t g = (size_t)x * Y + y;
          float sn, cs;
          sincosf(sc.phase[g] * fs, &sn, &cs);
          res = cmul(res, make_float2(cs, -sn));
          if (sc.amp != nullptr) {
            const float a = fminf(fmaxf(sc.amp[g], 1e-6f), 1.0f);
            res = cscale(res, exp2f(fs * log2f(a)));
          }
        }
        grow[y] = res;
      };
      if constexpr (PY::N2 == 32) {
        // lane b's inverse step-A outputs are y = b + 32 a: the epilogue runs
        // on them in registers, row by row (no store and reload of the row)
#pragma unroll 1
        for (int j = 0; j < RPW; ++j) {
          const int r = warp + NW * j;
          const int x = h * Xs + rank * R + r;
          const float2* row = buf + r * RS;
          float2* grow = p.spec + ((size_t)plane * X + x) * Y;
          const int b = lane;
          float2 v[PY::N1];
          v[0] = row[PY::pos(b)];
#pragma unroll
          for (int ka = 1; ka < PY::N1; ++ka) v[ka] = cmulc(row[PY::pos(b + 32 * ka)], tw_y[b * ka]);
          dft<PY::N1, true>(v);
          if (!epi) {
#pragma unroll
            for (int a = 0; a < PY::N1; ++a) grow[b + 32 * a] = v[a];
            continue;
          }
          float2 prev_last = make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < PY::N1; ++a) {
            float2 nxt = make_float2(0.f, 0.f);
            if (a + 1 < PY::N1 && sa) {
              nxt.x = __shfl_sync(0xffffffffu, v[a + 1 < PY::N1 ? a + 1 : a].x, 0);
              nxt.y = __shfl_sync(0xffffffffu, v[a + 1 < PY::N1 ? a + 1 : a].y, 0);
            }
            epilogue32(x, 32 * a, v[a], nxt, prev_last, grow);
          }
        }
      } else {
        for (int i = lane; i < RPW * PY::N2; i += 32) {
          const int j = i / PY::N2, b = i - j * PY::N2;
          stepA_inv_smem<PY>(buf + (warp + NW * j) * RS, b, tw_y);
        }
        __syncwarp();
#pragma unroll 1
        for (int j = 0; j < RPW; ++j) {
          const int r = warp + NW * j;
          const int x = h * Xs + rank * R + r;
          const float2* row = buf + r * RS;
          float2* grow = p.spec + ((size_t)plane * X + x) * Y;
          if (!epi) {
            for (int y = lane; y < Y; y += 32) grow[y] = row[PY::pos(y)];
            continue;
          }
          float2 prev_last = make_float2(0.f, 0.f);  // value at y0-1 (damped, not corrected)
          for (int y0 = 0; y0 < Y; y0 += 32) {
            const int y = y0 + lane;
            const float2 nxt = (lane == 31 && y + 1 < Y) ? row[PY::pos(y + 1)] : make_float2(0.f, 0.f);
            epilogue32(x, y0, row[PY::pos(y)], nxt, prev_last, grow);
          }
        }
      }
      __syncwarp();
    }
    // rows of a of my next plane, while the other warps finish
    if (plane + ncl < p.nplanes) {
      prefetch_rows(plane + ncl, 0);
      issued = (plane + ncl) * 2;
    }
  }
  cp_async_wait_all();
  // no bulk copy may still be landing in shared memory when the block exits
  if (row_pending) mbar_wait_bounded(&row_mbar[warp], row_phase, p.status);
}

// ---------------------------------------------------------------------------
bool asg_xy_l2_supported(int X, int Y, int nsub, int* G_out) {
  if (X % nsub) return false;
  const int Xs = X / nsub;
  int ok = 0;
  switch (Y) {
    case 128: ok = (Xs == 32 || Xs == 64); break;
    case 192: ok = (Xs == 96); break;
    case 256: ok = (Xs == 128); break;
    case 384: ok = (Xs == 192); break;
    case 512: ok = (Xs == 256); break;
    default: ok = 0;
  }
  if (!ok) return false;
  const int G = Xs / 16;
  if (G < 1 || G > 16 || Y % G) return false;
  if (G_out) *G_out = G;
  return true;
}

// Groups of G CTAs that a cooperative launch keeps resident at once.
template <class K>
static int coop_max_groups(K kern, int nt, size_t smem, int G) {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem) != cudaSuccess)
    return 0;
  return per_sm * nsm / G;
}

// Launches `units` (sub-)planes over at most `resident` groups (clusters, or
// CTA groups of a cooperative launch) and the scratch the plan sized.
template <class K>
static int launch_groups(K kern, const XYParams& p, cudaLaunchConfig_t cfg, int resident,
                         int units, cudaStream_t st) {
  int ng = resident < units ? resident : units;
  if (ng > p.l2_max_clusters) ng = p.l2_max_clusters;
  if (ng < 1) return ASG_ERR_SHAPE;
  cudaLaunchAttribute coop[1];
  if (p.coop) {
    if (p.grp_cnt == nullptr) return ASG_ERR_ARG;
    // every CTA of the grid is resident, so the counter barriers of a group
    // always complete
    if (cudaMemsetAsync(p.grp_cnt, 0, (size_t)ng * sizeof(unsigned), st) != cudaSuccess ||
        cudaMemsetAsync(p.grp_cnt + p.l2_max_clusters, 0, (size_t)ng * sizeof(unsigned), st) !=
            cudaSuccess)
      return ASG_ERR_CUDA;
    coop[0].id = cudaLaunchAttributeCooperative;
    coop[0].val.cooperative = 1;
    cfg.attrs = coop;
    cfg.numAttrs = 1;
  }
  cfg.gridDim = dim3(p.G * ng, 1, 1);
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, p);
  return e == cudaSuccess ? ASG_OK : ASG_ERR_CUDA;
}

// R rows per CTA and NT threads per block; the plan's group size p.G is that
// of 16-row CTAs (the cluster shape), the launch uses Xn / R.
template <int Yn, int Xn, int R, int NT>
static int launch_l2(const XYParams& pin, cudaStream_t st) {
  using PY = FastPlan<Yn>;
  using PX = FastPlan<Xn>;
  XYParams p = pin;
  if (p.G != Xn / 16) return ASG_ERR_SHAPE;
  p.G = Xn / R;
  const int Yc = Yn / p.G;
  const int nbuf = (R * PY::PADDED > Xn * Yc) ? R * PY::PADDED : Xn * Yc;
  p.l2_buf_elems = nbuf;
  const size_t smem =
      L2Shape<PY, NT>::kTablesInSmem
          ? (size_t)(nbuf + Yn + Xn) * sizeof(float2) + (size_t)(Yn + 2 * Xn) * sizeof(int)
          : (size_t)nbuf * sizeof(float2);
  auto kern = xy_l2<PY, PX, R, NT>;
  static int max_clusters_dev[ASG_MAX_DEVICES], cached_G_dev[ASG_MAX_DEVICES];
  static bool init_dev[ASG_MAX_DEVICES] = {};
  const int dev = asg_device_slot();
  int& max_clusters = max_clusters_dev[dev];
  int& cached_G = cached_G_dev[dev];
  if (!init_dev[dev]) {
    max_clusters = -1;
    cached_G = -1;
    init_dev[dev] = true;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static int max_groups_dev[ASG_MAX_DEVICES];
  int& max_groups = max_groups_dev[dev];
  if (max_clusters < 0 || cached_G != p.G) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return ASG_ERR_CUDA;
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cfg.gridDim = dim3(p.G * 1024, 1, 1);
    int n = 0;
    // groups of more than 16 CTAs run only as cooperative launches
    if (p.G > 16 || cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess || n <= 0)
      n = 1;
    max_clusters = n;
    max_groups = coop_max_groups(kern, NT, smem, p.G);
    cached_G = p.G;
  }
  const int nq = p.nplanes * p.nsub;
  return launch_groups(kern, p, cfg, p.coop ? max_groups : max_clusters, nq, st);
}

// Cooperative launches of the transform (not the power sums, which keep the
// summation order of the cluster shape) run 8-row CTAs of 4 warps from
// 256-wide planes up: 512 x 512 x 1024 xy_A/xy_B 1.33 -> 1.25 ms against
// 16-row CTAs of 8 warps (more blocks per SM to overlap each other's load
// waits; 4-row CTAs of 2 warps were slower again).  Thread-block clusters hold
// at most 16 CTAs and keep 16 rows per CTA.
template <int Yn, int Xn>
static int launch_l2_mode(const XYParams& p, cudaStream_t st) {
  if constexpr (Yn >= 256) {
    if (p.coop && !p.power_only && p.rows8) return launch_l2<Yn, Xn, 8, 128>(p, st);
  }
  return launch_l2<Yn, Xn, 16, 256>(p, st);
}

int asg_launch_xy_l2(const XYParams& p, cudaStream_t st) {
  const int Xs = p.X / p.nsub;
  switch (p.Y) {
    case 128: return Xs == 32 ? launch_l2_mode<128, 32>(p, st) : launch_l2_mode<128, 64>(p, st);
    case 192: return launch_l2_mode<192, 96>(p, st);
    case 256: return launch_l2_mode<256, 128>(p, st);
    case 384: return launch_l2_mode<384, 192>(p, st);
    case 512: return launch_l2_mode<512, 256>(p, st);
    default: return ASG_ERR_SHAPE;
  }
}

// ---------------------------------------------------------------------------
template <int Yn, int Xn>
static int launch_l2c(const XYParams& pin, cudaStream_t st) {
  using PY = FastPlan<Yn>;
  using PX = FastPlan<Xn>;
  constexpr int R = 16, NT = 256;
  constexpr int G = Xn / R, Yc = Yn / G, YR = Yc < 16 ? Yc : 16;
  XYParams p = pin;
  if (p.G != G || p.nsub != 2) return ASG_ERR_SHAPE;
  const int nbuf = (R * PY::PADDED > 2 * Xn * YR) ? R * PY::PADDED : 2 * Xn * YR;
  p.l2_buf_elems = nbuf;
  const size_t smem = (size_t)(nbuf + Yn + Xn) * sizeof(float2) +
                      (size_t)(2 * (2 * Xn) + 2 * Yn) * sizeof(float) +
                      (size_t)(Yn + 2 * Xn) * sizeof(int);
  auto kern = xy_l2c<PY, PX, R, NT>;
  static int max_clusters_dev[ASG_MAX_DEVICES];
  static bool init_dev[ASG_MAX_DEVICES] = {};
  const int dev = asg_device_slot();
  int& max_clusters = max_clusters_dev[dev];
  if (!init_dev[dev]) {
    max_clusters = -1;
    init_dev[dev] = true;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static int max_groups_dev[ASG_MAX_DEVICES];
  int& max_groups = max_groups_dev[dev];
  if (max_clusters < 0) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return ASG_ERR_CUDA;
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cfg.gridDim = dim3(G * 1024, 1, 1);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess || n <= 0) n = 1;
    max_clusters = n;
    max_groups = coop_max_groups(kern, NT, smem, G);
  }
  return launch_groups(kern, p, cfg, p.coop ? max_groups : max_clusters, p.nplanes, st);
}

int asg_launch_xy_l2_closing(const XYParams& p, cudaStream_t st) {
  const int Xs = p.X / p.nsub;
  switch (p.Y) {
    case 128: return Xs == 32 ? launch_l2c<128, 32>(p, st) : launch_l2c<128, 64>(p, st);
    case 192: return launch_l2c<192, 96>(p, st);
    case 256: return launch_l2c<256, 128>(p, st);
    case 384: return launch_l2c<384, 192>(p, st);
    case 512: return launch_l2c<512, 256>(p, st);
    default: return ASG_ERR_SHAPE;
  }
}
