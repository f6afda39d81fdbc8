// pm_setup.cpp -- host set-up of the 'mesh' macro (Main.f:481-870):
// equation numbering, node graph, node-panel matrix structure, element
// colouring and the element -> panel slot map, then upload to the device.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "pm_internal.h"

namespace pm {

namespace {

template <typename T>
int upload(Handle* h, T** dst, const T* src, size_t n) {
  if (n == 0) {
    *dst = nullptr;
    return PM_OK;
  }
  if (cudaMalloc((void**)dst, sizeof(T) * n) != cudaSuccess) {
    h->err = "cudaMalloc failed (" + std::to_string(sizeof(T) * n) + " bytes)";
    return PM_E_NOMEM;
  }
  if (src && cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    h->err = "cudaMemcpy failed";
    return PM_E_CUDA;
  }
  return PM_OK;
}

}  // namespace

int build_structure(Handle* h, const int32_t* ix, const int32_t* idflag,
                    const int32_t* fnno, const double* x, const int32_t* num) {
  const int nnode = h->nnode, numel = h->numel, nen = h->nen, nenv = h->nenv;
  const int ndf = kNdf;
  // ---- equation numbering: numeqpmec2 (Numeq.f:86-151) ---------------------
  // Nodes are visited in num order; each free dof of the visited node takes
  // the next equation number; the pressure dof exists on vertex nodes only.
  h->h_eq.assign((size_t)ndf * nnode, 0);
  int neq = 0;
  for (int i = 0; i < nnode; ++i) {
    const int n = num ? num[i] : i + 1;
    if (n < 1 || n > nnode) {
      h->err = "num: node id out of range";
      return PM_E_ARG;
    }
    const int ndfn = (fnno[n - 1] == 1) ? ndf : ndf - 1;
    for (int j = 0; j < ndfn; ++j)
      if (idflag[(size_t)ndf * (n - 1) + j] == 0) h->h_eq[(size_t)ndf * (n - 1) + j] = ++neq;
  }
  h->neq = neq;
  if (neq == 0) {
    h->err = "no free equations";
    return PM_E_ARG;
  }
  // first equation (0-based) and free-dof count per node
  std::vector<int32_t> e0(nnode, -1), dn(nnode, 0);
  for (int n = 0; n < nnode; ++n) {
    int lo = 0x7fffffff, c = 0;
    for (int j = 0; j < ndf; ++j) {
      const int e = h->h_eq[(size_t)ndf * n + j];
      if (e > 0) {
        lo = std::min(lo, e - 1);
        ++c;
      }
    }
    dn[n] = c;
    e0[n] = c ? lo : -1;
  }
  // ---- node -> element incidence -------------------------------------------
  std::vector<int64_t> inc_ptr(nnode + 1, 0);
  for (int el = 0; el < numel; ++el)
    for (int k = 0; k < nen; ++k) {
      const int n = ix[(size_t)(nen + 1) * el + k];
      if (n < 1 || n > nnode) {
        h->err = "ix: node id out of range in element " + std::to_string(el + 1);
        return PM_E_ARG;
      }
      inc_ptr[n]++;
    }
  for (int n = 0; n < nnode; ++n) inc_ptr[n + 1] += inc_ptr[n];
  std::vector<int32_t> inc(inc_ptr[nnode]);
  {
    std::vector<int64_t> pos(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int el = 0; el < numel; ++el)
      for (int k = 0; k < nen; ++k) inc[pos[ix[(size_t)(nen + 1) * el + k] - 1]++] = el;
  }
  // ---- node graph (graph_v1, Graph.f:72-133) restricted to free nodes ------
  // neighbours of I: every node sharing an element with I, I included,
  // ordered by first equation; colpos = position of their first column.
  std::vector<int64_t> nb_ptr(nnode + 1, 0);
  auto neighbours = [&](int n, std::vector<int32_t>& buf) {
    buf.clear();
    for (int64_t k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) {
      const int el = inc[k];
      for (int a = 0; a < nen; ++a) {
        const int m = ix[(size_t)(nen + 1) * el + a] - 1;
        if (dn[m] > 0) buf.push_back(m);
      }
    }
    std::sort(buf.begin(), buf.end(), [&](int a, int b) { return e0[a] < e0[b]; });
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
#pragma omp parallel
  {
    std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 1024)
    for (int n = 0; n < nnode; ++n) {
      if (dn[n] == 0) continue;
      neighbours(n, buf);
      nb_ptr[n + 1] = (int64_t)buf.size();
    }
  }
  for (int n = 0; n < nnode; ++n) nb_ptr[n + 1] += nb_ptr[n];
  std::vector<int32_t> nb(nb_ptr[nnode]), nb_pos(nb_ptr[nnode]);
  std::vector<int32_t> Wn(nnode, 0), lown(nnode, 0);
#pragma omp parallel
  {
    std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 1024)
    for (int n = 0; n < nnode; ++n) {
      if (dn[n] == 0) continue;
      neighbours(n, buf);
      int pos = 0, low = -1;
      for (size_t k = 0; k < buf.size(); ++k) {
        nb[nb_ptr[n] + k] = buf[k];
        nb_pos[nb_ptr[n] + k] = pos;
        if (buf[k] == n) low = pos;
        pos += dn[buf[k]];
      }
      Wn[n] = pos;
      lown[n] = low;
    }
  }
  // ---- active nodes in equation order ----------------------------------------
  std::vector<int32_t> act;
  for (int n = 0; n < nnode; ++n)
    if (dn[n] > 0) act.push_back(n);
  std::sort(act.begin(), act.end(), [&](int a, int b) { return e0[a] < e0[b]; });
  const int nact = (int)act.size();
  h->h_eq0.resize(nact);
  h->h_d.resize(nact);
  h->h_W.resize(nact);
  h->h_low.resize(nact);
  h->h_val_off.resize(nact + 1);
  h->h_col_off.resize(nact + 1);
  std::vector<int64_t> node_val_off(nnode, -1);
  std::vector<int32_t> node_W(nnode, 0);
  int64_t vo = 0, co = 0, nad = 0;
  for (int k = 0; k < nact; ++k) {
    const int n = act[k];
    h->h_eq0[k] = e0[n];
    h->h_d[k] = dn[n];
    h->h_W[k] = Wn[n];
    h->h_low[k] = lown[n];
    node_W[n] = Wn[n];
    for (int q = 0; q < dn[n]; ++q) nad += lown[n] + q;
  }
  // SpMV visiting order: by free dofs, then panel width (descending), then
  // equation order, so the nodes sharing a warp run identical loops.  The
  // panels and their column lists are stored in this order, so the SpMV
  // streams them sequentially (a scattered visit over GBs of panels costs
  // DRAM pages and TLB reach).
  // For a batch of meshes the instance comes first, so that an instance's
  // nodes are contiguous in the order and a converged instance's panels are
  // skipped as one stretch.
  std::vector<int32_t> order(nact), inst_act(nact, 0);
  if (h->ninst > 0)
    for (int k = 0; k < nact; ++k)
      inst_act[k] = (int32_t)(std::upper_bound(h->h_inst_node.begin(), h->h_inst_node.end(),
                                               act[k]) -
                              h->h_inst_node.begin()) - 1;
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (inst_act[a] != inst_act[b]) return inst_act[a] < inst_act[b];
    if (h->h_d[a] != h->h_d[b]) return h->h_d[a] > h->h_d[b];
    return h->h_W[a] > h->h_W[b];
  });
  h->h_inst_act = inst_act;
  for (int i = 0; i < nact; ++i) {
    const int k = order[i];
    const int n = act[k];
    h->h_val_off[k] = vo;
    h->h_col_off[k] = co;
    node_val_off[n] = vo;
    vo += (int64_t)dn[n] * Wn[n];
    co += Wn[n];
  }
  h->h_val_off[nact] = vo;
  h->h_col_off[nact] = co;
  h->nad = nad;
  h->h_cols.resize(co);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int k = 0; k < nact; ++k) {
    const int n = act[k];
    int64_t c = h->h_col_off[k];
    for (int64_t j = nb_ptr[n]; j < nb_ptr[n + 1]; ++j) {
      const int m = nb[j];
      for (int q = 0; q < dn[m]; ++q) h->h_cols[c++] = e0[m] + q;
    }
  }
  // ---- element colouring (semantics of Colormsh.f:160-254): greedy in element
  // order, no two elements of one colour share a vertex --------------------
  std::vector<int32_t> colour(numel, -1);
  {
    std::vector<std::vector<int32_t>> ncol(nnode);
    int ncolours = 0;
    std::vector<char> used;
    for (int el = 0; el < numel; ++el) {
      used.assign(ncolours + 1, 0);
      for (int k = 0; k < nenv; ++k)
        for (int c : ncol[ix[(size_t)(nen + 1) * el + k] - 1]) used[c] = 1;
      int c = 0;
      while (c < ncolours && used[c]) ++c;
      if (c == ncolours) ++ncolours;
      colour[el] = c;
      for (int k = 0; k < nenv; ++k) ncol[ix[(size_t)(nen + 1) * el + k] - 1].push_back(c);
    }
    h->numcolors = ncolours;
  }
  h->color_ptr.assign(h->numcolors + 1, 0);
  for (int el = 0; el < numel; ++el) h->color_ptr[colour[el] + 1]++;
  for (int c = 0; c < h->numcolors; ++c) h->color_ptr[c + 1] += h->color_ptr[c];
  std::vector<int32_t> celems(numel);
  {
    std::vector<int32_t> pos(h->color_ptr.begin(), h->color_ptr.end() - 1);
    for (int el = 0; el < numel; ++el) celems[pos[colour[el]]++] = el + 1;
  }
  // ---- slot map: column position of node b's dofs in node a's panel ------------
  std::vector<int32_t> slot((size_t)nen * nen * numel, -1);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < numel; ++k) {
    const int el = celems[k] - 1;
    const int32_t* nodes = &ix[(size_t)(nen + 1) * el];
    for (int a = 0; a < nen; ++a) {
      const int na = nodes[a] - 1;
      if (dn[na] == 0) continue;
      const int32_t* lst = &nb[nb_ptr[na]];
      const int64_t len = nb_ptr[na + 1] - nb_ptr[na];
      for (int b = 0; b < nen; ++b) {
        const int nbn = nodes[b] - 1;
        if (dn[nbn] == 0) continue;
        const int32_t* it = std::lower_bound(lst, lst + len, nbn, [&](int32_t u, int32_t v) {
          return e0[u] < e0[v];
        });
        slot[(size_t)nen * nen * k + (size_t)a * nen + b] = nb_pos[nb_ptr[na] + (it - lst)];
      }
    }
  }
  // ---- per-equation kind (cal_residuo_pm splits u and p) ---------------------
  std::vector<int32_t> kind(neq, 0);
  for (int n = 0; n < nnode; ++n) {
    const int e = h->h_eq[(size_t)ndf * n + 3];
    if (e > 0) kind[e - 1] = 1;
  }
  // ---- upload ------------------------------------------------------------------
  Panels& P = h->P;
  P.nact = nact;
  P.nnz = vo;
  P.ncols = co;
  int st;
  h->h_order = order;
  if ((st = upload(h, &P.order, order.data(), nact))) return st;
  if ((st = upload(h, &P.eq0, h->h_eq0.data(), nact))) return st;
  if ((st = upload(h, &P.d, h->h_d.data(), nact))) return st;
  if ((st = upload(h, &P.W, h->h_W.data(), nact))) return st;
  if ((st = upload(h, &P.low, h->h_low.data(), nact))) return st;
  if ((st = upload(h, &P.val_off, h->h_val_off.data(), nact))) return st;
  if ((st = upload(h, &P.col_off, h->h_col_off.data(), nact))) return st;
  if ((st = upload(h, &P.cols, h->h_cols.data(), (size_t)co))) return st;
  if ((st = upload(h, &P.node_val_off, node_val_off.data(), nnode))) return st;
  if ((st = upload(h, &P.node_W, node_W.data(), nnode))) return st;
  if ((st = upload<double>(h, &P.val, nullptr, (size_t)vo))) return st;
  if ((st = upload(h, &h->D.ix, ix, (size_t)(nen + 1) * numel))) return st;
  if ((st = upload(h, &h->D.eq, h->h_eq.data(), h->h_eq.size()))) return st;
  if ((st = upload(h, &h->D.x, x, (size_t)3 * nnode))) return st;
  if ((st = upload(h, &h->D.slot, slot.data(), slot.size()))) return st;
  if ((st = upload(h, &h->D.color_elems, celems.data(), celems.size()))) return st;
  if ((st = upload(h, &h->D.dofkind, kind.data(), kind.size()))) return st;
  if ((st = upload(h, &h->D.fnno, fnno, (size_t)nnode))) return st;
  h->h_fnno.assign(fnno, fnno + nnode);
  return build_meta(h, nullptr);
}

int build_meta(Handle* h, const int32_t* inst) {
  Panels& P = h->P;
  if (P.meta) {
    cudaFree(P.meta);
    P.meta = nullptr;
  }
  const int nact = P.nact;
  if (nact == 0 || P.nnz >= (int64_t(1) << 32) || P.ncols >= (int64_t(1) << 32)) return PM_OK;
  std::vector<int4> m(nact);
  for (int s = 0; s < nact; ++s) {
    const int k = h->h_order[s];
    const int W = h->h_W[k], d = h->h_d[k], in = inst ? inst[k] : 0;
    if (W >= 8192 || d > 7 || in >= 65536) return PM_OK;
    const uint32_t dw = (uint32_t)d | ((uint32_t)W << 3) | ((uint32_t)in << 16);
    m[s] = make_int4(h->h_eq0[k], (int)dw, (int)(uint32_t)h->h_val_off[k],
                     (int)(uint32_t)h->h_col_off[k]);
  }
  return upload(h, &P.meta, m.data(), (size_t)nact);
}

// Offsets of the node records of the compensated operator (layout in
// CompVals): 16-byte aligned, in the SpMV visiting order; the records
// themselves are written on the device from the FP64 panels.
int build_rec_layout(Handle* h) {
  Panels& P = h->P;
  const int nact = P.nact;
  std::vector<int64_t> off(nact > 0 ? nact : 1, 0);
  int64_t o = 0;
  int rmax = 16;
  for (int i = 0; i < nact; ++i) {
    const int k = h->h_order[i];
    const int d = h->h_d[k], Wp = (h->h_W[k] + 3) & ~3;
    const int R = 4 * d * Wp + ((d * Wp + 15) & ~15) + 4 * Wp;
    off[k] = o;
    o += R;
    if (R > rmax) rmax = R;
  }
  int st;
  if ((st = upload(h, &P.rec_off, off.data(), off.size()))) return st;
  if ((st = upload<uint8_t>(h, &P.rec, nullptr, (size_t)(o > 0 ? o : 16)))) return st;
  P.rec_max = rmax;
  if (ca_configure(rmax, &P.ca_warps, &P.ca_grid) != cudaSuccess) {
    h->err = "record SpMV set-up failed";
    return PM_E_CUDA;
  }
  // streamed record kernel: batches of up to kCsNodes consecutive records
  // (one warp per node), a stage holds the largest batch
  const int stage_bytes = kCsNodes * rmax;
  int nstage = 0, ctas = 0, sms = 0, dev = 0;
  if (cs_configure(stage_bytes, &nstage, &ctas) != cudaSuccess ||
      cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    h->err = "streamed SpMV set-up failed";
    return PM_E_CUDA;
  }
  sms *= ctas;
  if (nstage >= 2 && nact > 0) {
    std::vector<int4> desc(nact);
    std::vector<int32_t> bslot, bbytes;
    std::vector<int64_t> boff;
    int64_t total = 0;
    for (int i = 0; i < nact;) {
      const int k0 = h->h_order[i];
      const int64_t start = off[k0];
      int j = i, bytes = 0;
      while (j < nact && j - i < kCsNodes) {
        const int k = h->h_order[j];
        const int Wp = (h->h_W[k] + 3) & ~3;
        const int R = 4 * h->h_d[k] * Wp + ((h->h_d[k] * Wp + 15) & ~15) + 4 * Wp;
        desc[j] = make_int4(h->h_eq0[k], h->h_d[k], h->h_W[k], (int)(off[k] - start));
        bytes += R;
        ++j;
      }
      bslot.push_back(i);
      boff.push_back(start);
      bbytes.push_back(bytes);
      total += bytes;
      i = j;
    }
    const int nb = (int)bslot.size();
    bslot.push_back(nact);
    // runs of batches per CTA, balanced by estimated time: a batch costs its
    // bytes at the CTA's share of HBM plus a fixed part (the gather latency
    // and the stage hand-over, about the time of 24 KB), so that CTAs with
    // many small boundary-node batches do not set the kernel's duration
    const int64_t kFixed = 24 * 1024;
    int64_t cost_total = total + kFixed * (int64_t)nb;
    const int grid = std::max(1, std::min(sms, nb));
    std::vector<int32_t> cta(grid + 1, nb);
    cta[0] = 0;
    int64_t acc = 0;
    int c = 1;
    for (int b = 0; b < nb && c < grid; ++b) {
      acc += bbytes[b] + kFixed;
      while (c < grid && acc * grid >= cost_total * c) cta[c++] = b + 1;
    }
    for (; c < grid; ++c) cta[c] = nb;
    if ((st = upload(h, &P.cs_desc, desc.data(), desc.size()))) return st;
    if ((st = upload(h, &P.cs_batch_slot, bslot.data(), bslot.size()))) return st;
    if ((st = upload(h, &P.cs_batch_off, boff.data(), boff.size()))) return st;
    if ((st = upload(h, &P.cs_batch_bytes, bbytes.data(), bbytes.size()))) return st;
    if ((st = upload(h, &P.cs_cta_batch, cta.data(), cta.size()))) return st;
    if ((st = upload<int>(h, &P.fault, nullptr, 1))) return st;
    if (cudaMemset(P.fault, 0, sizeof(int)) != cudaSuccess) {
      h->err = "cudaMemset failed";
      return PM_E_CUDA;
    }
    P.cs_grid = grid;
    P.cs_nstage = nstage;
    P.cs_stage_bytes = stage_bytes;
    if (getenv("PM_DEBUG"))
      fprintf(stderr, "streamed SpMV: %d batches, %d CTAs (%d per SM), %d stages of %d bytes\n",
              nb, grid, ctas, nstage, stage_bytes);
  }
  return PM_OK;
}

}  // namespace pm
