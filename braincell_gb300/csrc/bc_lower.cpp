// One-time lowering of a cell: branch geometry -> CVs -> point tree -> axial
// coefficients.  Follows the reference's declaration-time pipeline:
//   CV geometry        _discretization/geometry.py:214-434 (frusta, area, axial
//                      factor, midpoint split), :614-736 (per-CV assembly)
//   half resistances   _discretization/base.py:530-559 (R = Ra * factor)
//   point tree         _discretization/node_build.py:58-285, :352-371, :436-449
//   edge conductance   quad/_staggered.py:546-576 (series halves on one branch,
//                      parallel otherwise)
//   row capacitance    quad/_staggered.py:579-593 (dummy 1 uF on boundary rows)
//   axial operator     quad/_staggered.py:360-390 (coefficients g/C in ms^-1)
#include <cmath>
#include <map>
#include <string>
#include <utility>

#include "bc_internal.h"

namespace bc {
namespace {

constexpr double kEpsParam = 1e-9;
constexpr double kEpsLen = 1e-6;
constexpr double kPi = 3.14159265358979323846;

struct Piece {
  double prox, dist, len, r0, r1;
};

// Clip the branch's segments to the normalised interval [prox, dist].
bool build_frusta(const double* L, const double* rp, const double* rd, int64_t nseg, double prox, double dist,
                  std::vector<Piece>& out, std::string& err) {
  out.clear();
  double total = 0.0;
  for (int64_t i = 0; i < nseg; ++i) total += L[i];
  if (total <= kEpsLen) {
    err = "branch total length must be > 1e-6 um";
    return false;
  }
  const double start = prox * total, end = dist * total;
  double s0 = 0.0;
  for (int64_t i = 0; i < nseg; ++i) {
    const double seg = L[i], s1 = s0 + seg;
    if (rp[i] <= 0.0 || rd[i] <= 0.0) {
      err = "all branch radii must be > 0";
      return false;
    }
    if (seg <= kEpsLen) {
      // zero-length radius jump: kept by the CV that owns its position
      const bool same = std::fabs(rp[i] - rd[i]) <= 1e-8 + 1e-5 * std::fabs(rd[i]);
      bool owns = !(s0 < start - kEpsLen || s0 > end + kEpsLen);
      if (owns && s0 <= start + kEpsLen) owns = start <= kEpsLen;
      if (!same && owns) {
        const double xj = std::max(prox, std::min(dist, s0 / total));
        out.push_back({xj, xj, 0.0, rp[i], rd[i]});
      }
      s0 = s1;
      continue;
    }
    const double left = std::max(s0, start), right = std::min(s1, end);
    if (right - left > kEpsLen) {
      const double t0 = (left - s0) / seg, t1 = (right - s0) / seg;
      const double r0 = rp[i] + (rd[i] - rp[i]) * t0;
      const double r1 = rp[i] + (rd[i] - rp[i]) * t1;
      const double x0 = std::max(prox, std::min(dist, left / total));
      const double x1 = std::max(prox, std::min(dist, right / total));
      out.push_back({x0, x1, right - left, r0, r1});
    }
    s0 = s1;
  }
  if (out.empty()) {
    err = "CV produced no frusta";
    return false;
  }
  return true;
}

double lateral_area(const std::vector<Piece>& f) {
  double a = 0.0;
  for (const Piece& p : f) a += kPi * (p.r0 + p.r1) * std::sqrt(p.len * p.len + (p.r1 - p.r0) * (p.r1 - p.r0));
  return a;
}

double axial_factor(const std::vector<Piece>& f) {
  double s = 0.0;
  for (const Piece& p : f) s += (p.len * 1e-4) / (kPi * (p.r0 * 1e-4) * (p.r1 * 1e-4));
  return s;
}

void split(const std::vector<Piece>& f, double x, std::vector<Piece>& left, std::vector<Piece>& right) {
  left.clear();
  right.clear();
  for (const Piece& p : f) {
    if (p.dist <= x + kEpsParam) {
      left.push_back(p);
      continue;
    }
    if (p.prox >= x - kEpsParam) {
      right.push_back(p);
      continue;
    }
    const double span = p.dist - p.prox;
    if (span <= kEpsParam) continue;
    const double ratio = std::max(0.0, std::min(1.0, (x - p.prox) / span));
    const double ll = p.len * ratio, lr = p.len - ll;
    const double rm = p.r0 + (p.r1 - p.r0) * ratio;
    if (ll > kEpsLen) left.push_back({p.prox, x, ll, p.r0, rm});
    if (lr > kEpsLen) right.push_back({x, p.dist, lr, rm, p.r1});
  }
}

}  // namespace

// CV ids of a branch are contiguous: first_cv[b] .. first_cv[b] + ncv[b] - 1.
static void branch_first_cv(const bc_batch_spec& s, int64_t c, std::vector<int32_t>& first) {
  const int64_t b0 = s.cell_branch_offsets[c], b1 = s.cell_branch_offsets[c + 1];
  first.resize(b1 - b0);
  int32_t acc = 0;
  for (int64_t b = b0; b < b1; ++b) {
    first[b - b0] = acc;
    acc += s.branch_ncv[b];
  }
}

// Owning CV (branch-local index) of normalised coordinate x under a uniform tiling.
static int32_t locate_cv_local(int32_t ncv, double x) {
  if (x <= kEpsParam) return 0;
  if (x >= 1.0 - kEpsParam) return ncv - 1;
  for (int32_t k = 0; k < ncv; ++k) {
    const double prox = double(k) / ncv, dist = double(k + 1) / ncv;
    if (prox - kEpsParam <= x && x < dist - kEpsParam) return k;
  }
  for (int32_t k = 0; k < ncv; ++k)
    if (std::fabs(x - double(k + 1) / ncv) <= kEpsParam) return k;
  return ncv - 1;
}

bc_status lower_cell(const bc_batch_spec& s, int64_t c, LoweredCell& out) {
  const int64_t b0 = s.cell_branch_offsets[c], b1 = s.cell_branch_offsets[c + 1];
  const int32_t nb = int32_t(b1 - b0);
  if (nb <= 0) return fail(BC_ERR_INVALID, "cell " + std::to_string(c) + " has no branches");
  if (s.branch_parent[b0] != -1)
    return fail(BC_ERR_INVALID, "cell " + std::to_string(c) + ": branch 0 must be the root (parent -1)");
  std::vector<int32_t> first;
  branch_first_cv(s, c, first);
  int32_t n_cv = 0;
  for (int64_t b = b0; b < b1; ++b) {
    if (s.branch_ncv[b] < 1) return fail(BC_ERR_INVALID, "branch_ncv must be >= 1");
    n_cv += s.branch_ncv[b];
  }
  out = LoweredCell();
  out.n_cv = n_cv;
  out.cv_area.resize(n_cv);
  std::vector<double> r_prox(n_cv), r_dist(n_cv), cap(n_cv);
  std::vector<int32_t> cv_branch(n_cv), cv_region(n_cv);
  std::vector<Piece> fr, left, right;
  std::string err;
  // ------------------------------------------------ CV geometry
  for (int32_t lb = 0; lb < nb; ++lb) {
    const int64_t b = b0 + lb;
    const int32_t region = s.branch_region[b];
    if (region < 0 || region >= s.n_regions) return fail(BC_ERR_INVALID, "branch_region out of range");
    const int64_t rc = c * s.n_regions + region;
    const double ra = s.region_ra[rc], cm = s.region_cm[rc];
    if (!(ra > 0.0) || !(cm > 0.0)) return fail(BC_ERR_INVALID, "region cm and Ra must be > 0");
    const int64_t g0 = s.branch_seg_offsets[b], g1 = s.branch_seg_offsets[b + 1];
    if (g1 <= g0) return fail(BC_ERR_INVALID, "branch has no segments");
    const int32_t n = s.branch_ncv[b];
    for (int32_t k = 0; k < n; ++k) {
      const double prox = double(k) / n, dist = double(k + 1) / n;
      if (!build_frusta(s.seg_length + g0, s.seg_r_prox + g0, s.seg_r_dist + g0, g1 - g0, prox, dist, fr, err))
        return fail(BC_ERR_INVALID, "cell " + std::to_string(c) + " branch " + std::to_string(lb) + ": " + err);
      const int32_t cv = first[lb] + k;
      const double area = lateral_area(fr);
      split(fr, 0.5 * (prox + dist), left, right);
      r_prox[cv] = ra * (left.empty() ? 0.0 : axial_factor(left));
      r_dist[cv] = ra * (right.empty() ? 0.0 : axial_factor(right));
      out.cv_area[cv] = area;
      cap[cv] = area * 1e-8 * cm * 1e-6;  // F
      cv_branch[cv] = lb;
      cv_region[cv] = region;
    }
  }
  // ------------------------------------------------ point tree
  // endpoint[(branch, side)] -> node; side 0 = x 0, 1 = x 1
  std::vector<int32_t> endpoint(size_t(nb) * 2, -1);
  std::vector<int32_t> cv_mid(n_cv, -1);
  std::vector<int32_t> node_cv;  // -1 boundary
  std::vector<int32_t> node_vcv;  // a CV whose V_rest initialises the node
  // edges keyed by (parent, child) -> roles (cv, half: 0 prox / 1 dist); creation order kept
  std::vector<std::pair<int32_t, int32_t>> edge_key;
  std::vector<std::vector<std::pair<int32_t, int32_t>>> edge_roles;
  std::map<std::pair<int32_t, int32_t>, int32_t> edge_index;
  auto new_node = [&](int32_t cv, bool mid) {
    node_cv.push_back(mid ? cv : -1);
    node_vcv.push_back(cv);
    return int32_t(node_cv.size() - 1);
  };
  auto add_edge = [&](int32_t p, int32_t ch, int32_t cv, int32_t half) {
    auto key = std::make_pair(p, ch);
    auto it = edge_index.find(key);
    int32_t e;
    if (it == edge_index.end()) {
      e = int32_t(edge_key.size());
      edge_index.emplace(key, e);
      edge_key.push_back(key);
      edge_roles.emplace_back();
    } else {
      e = it->second;
    }
    for (auto& r : edge_roles[e])
      if (r.first == cv && r.second == half) return;
    edge_roles[e].push_back({cv, half});
  };
  const int32_t root = new_node(first[0], false);
  endpoint[0] = root;
  std::vector<int32_t> order;
  for (int32_t lb = 0; lb < nb; ++lb) {
    const int64_t b = b0 + lb;
    const int32_t n = s.branch_ncv[b];
    int32_t att;
    double ax;
    if (lb == 0) {
      att = root;
      ax = 0.0;
    } else {
      const int32_t pb = s.branch_parent[b];
      if (pb < 0 || pb >= lb)
        return fail(BC_ERR_INVALID, "cell " + std::to_string(c) + ": branch parents must precede children");
      const double px = s.branch_parent_x[b];
      if (px <= kEpsParam) {
        att = endpoint[size_t(pb) * 2 + 0];
      } else if (px >= 1.0 - kEpsParam) {
        att = endpoint[size_t(pb) * 2 + 1];
      } else {
        att = cv_mid[first[pb] + locate_cv_local(s.branch_ncv[b0 + pb], px)];
      }
      if (att < 0) return fail(BC_ERR_INVALID, "unresolved attachment node");
      ax = s.branch_child_x[b];
    }
    const bool fwd = ax <= kEpsParam;
    order.resize(n);
    for (int32_t k = 0; k < n; ++k) order[k] = fwd ? first[lb] + k : first[lb] + (n - 1 - k);
    const int32_t entry = fwd ? 0 : 1, exit_half = fwd ? 1 : 0;
    endpoint[size_t(lb) * 2 + (fwd ? 0 : 1)] = att;
    for (int32_t k = 0; k < n; ++k) cv_mid[order[k]] = new_node(order[k], true);
    const int32_t term = new_node(order[n - 1], false);
    endpoint[size_t(lb) * 2 + (fwd ? 1 : 0)] = term;
    for (int32_t k = 0; k < n; ++k) {
      const int32_t mid = cv_mid[order[k]];
      const int32_t par = k == 0 ? att : cv_mid[order[k - 1]];
      const int32_t chi = k == n - 1 ? term : cv_mid[order[k + 1]];
      add_edge(par, mid, order[k], entry);
      add_edge(mid, chi, order[k], exit_half);
    }
  }
  const int32_t nn = int32_t(node_cv.size());
  out.n_node = nn;
  out.parent.assign(nn, -1);
  out.alpha.assign(nn, 0.0);
  out.beta.assign(nn, 0.0);
  out.diag.assign(nn, 0.0);
  out.region.assign(nn, -1);
  out.node_vrest.assign(nn, 0.0);
  std::vector<double> rowcap(nn, 1e-6);  // F; 1 uF dummy on boundary rows
  for (int32_t i = 0; i < nn; ++i) {
    if (node_cv[i] >= 0) {
      rowcap[i] = cap[node_cv[i]];
      out.region[i] = cv_region[node_cv[i]];
    }
    const int32_t vr = cv_region[node_vcv[i]];
    out.node_vrest[i] = s.region_params[(c * s.n_regions + vr) * BC_NPARAM + BC_P_VREST];
  }
  for (size_t e = 0; e < edge_key.size(); ++e) {
    const int32_t p = edge_key[e].first, ch = edge_key[e].second;
    if (out.parent[ch] != -1) return fail(BC_ERR_INVALID, "point tree node with two parents");
    out.parent[ch] = p;
    const auto& roles = edge_roles[e];
    double g;
    bool same_branch = true;
    for (auto& r : roles) same_branch = same_branch && cv_branch[r.first] == cv_branch[roles[0].first];
    if (roles.size() > 1 && same_branch) {
      double rsum = 0.0;
      for (auto& r : roles) rsum += r.second == 0 ? r_prox[r.first] : r_dist[r.first];
      g = 1.0 / rsum;
    } else {
      g = 0.0;
      for (auto& r : roles) g += 1.0 / (r.second == 0 ? r_prox[r.first] : r_dist[r.first]);
    }
    if (!std::isfinite(g) || g <= 0.0) return fail(BC_ERR_INVALID, "non-positive axial conductance");
    const double pc = g / rowcap[p] * 1e-3, cc = g / rowcap[ch] * 1e-3;  // ms^-1
    out.diag[p] += pc;
    out.diag[ch] += cc;
    out.alpha[ch] = cc;  // A[child, parent] = -alpha
    out.beta[ch] = pc;   // A[parent, child] = -beta
  }
  out.cv_node = cv_mid;
  return BC_OK;
}

int32_t locate_node(const bc_batch_spec& s, int64_t c, const LoweredCell& lc, int32_t branch, double x) {
  // Re-derive the endpoint / midpoint the same way the tree was built.
  const int64_t b0 = s.cell_branch_offsets[c];
  const int32_t nb = int32_t(s.cell_branch_offsets[c + 1] - b0);
  if (branch < 0 || branch >= nb) return -1;
  std::vector<int32_t> first;
  branch_first_cv(s, c, first);
  const int32_t n = s.branch_ncv[b0 + branch];
  if (x > kEpsParam && x < 1.0 - kEpsParam) return lc.cv_node[first[branch] + locate_cv_local(n, x)];
  // endpoint: walk the construction again to find endpoint nodes
  std::vector<int32_t> endpoint(size_t(nb) * 2, -1);
  endpoint[0] = 0;
  int32_t next_id = 1;
  std::vector<int32_t> mid_of_cv(lc.n_cv, -1);
  for (int32_t lb = 0; lb < nb; ++lb) {
    const int64_t b = b0 + lb;
    const int32_t nc = s.branch_ncv[b];
    int32_t att;
    double ax;
    if (lb == 0) {
      att = 0;
      ax = 0.0;
    } else {
      const int32_t pb = s.branch_parent[b];
      const double px = s.branch_parent_x[b];
      if (px <= kEpsParam)
        att = endpoint[size_t(pb) * 2];
      else if (px >= 1.0 - kEpsParam)
        att = endpoint[size_t(pb) * 2 + 1];
      else
        att = mid_of_cv[first[pb] + locate_cv_local(s.branch_ncv[b0 + pb], px)];
      ax = s.branch_child_x[b];
    }
    const bool fwd = ax <= kEpsParam;
    endpoint[size_t(lb) * 2 + (fwd ? 0 : 1)] = att;
    for (int32_t k = 0; k < nc; ++k) mid_of_cv[fwd ? first[lb] + k : first[lb] + (nc - 1 - k)] = next_id++;
    endpoint[size_t(lb) * 2 + (fwd ? 1 : 0)] = next_id++;
  }
  return endpoint[size_t(branch) * 2 + (x <= kEpsParam ? 0 : 1)];
}

}  // namespace bc
