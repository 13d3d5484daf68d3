// Internal data model of the GB300 polarization library.
//
// One `System` mirrors the reference's ommp_system for the polarization path
// (src/mod_mmpol.F90:20-44, src/mod_electrostatics.F90:23-241): host copies
// of the topology and parameters, the device-resident arrays the kernels use,
// and the solver state (E_M2D cache, induced dipoles, warm-start flags).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace ommp {

// Constants of the reference (config/openmmpol_const.h.in, mod_constants.F90).
constexpr double kAng2Au = 1.8897261245650;
constexpr double kEpsRp = 2.220446049250313e-16 * 100.0;
constexpr int kSolverNone = 0, kSolverCG = 1, kSolverDIIS = 2, kSolverInversion = 3;
constexpr int kMatvNone = 0, kMatvIncore = 1, kMatvDirect = 2;
constexpr int kPrecFP64 = 0, kPrecMixed = 1, kPrecMixedDS = 2;

// Compressed sparse rows, 0-based.
struct Csr {
  int n = 0;
  std::vector<int> ri{0};
  std::vector<int> ci;
  int row_len(int i) const { return ri[i + 1] - ri[i]; }
  bool has(int i, int j) const {
    for (int k = ri[i]; k < ri[i + 1]; ++k)
      if (ci[k] == j) return true;
    return false;
  }
};

// Host-side description of a polarizable system, in atomic units.
struct HostModel {
  bool amoeba = false;
  int mm = 0, npol = 0, ld_cart = 1, n_ipd = 1;
  std::vector<double> cmm;          // [mm][3]
  std::vector<double> q0, q;        // [mm][ld_cart]; q is the lab-frame set
  std::vector<double> pol;          // [npol]
  std::vector<int> polar_mm;        // [npol]
  std::vector<int> mm_polar;        // [mm], -1 if not polarizable
  std::vector<double> thole;        // [mm]
  std::vector<double> damping;      // [npol] Thole 'a' (AMOEBA)
  double thole_scale = 0.0;
  std::vector<int> grp;             // [mm] polarization group (AMOEBA)
  int ngrp = 0;
  std::vector<int> frame, iz, ix, iy;  // [mm], -1 = none
  Csr conn[4];                      // atoms at 1, 2, 3, 4 bonds
  Csr grp_atoms;                    // group -> atoms
  Csr pg_conn[4];                   // groups: same, 1, 2, 3 links apart
  double mscale[4], pscale[4], dscale[4], uscale[4], pscale_intra[4];
  bool fmm_requested = false;       // reference would auto-enable FMM (> 1000 atoms)
};

// Scaled pairs, target-major: for target row t, entries (source, scale).
struct ScaledPairs {
  std::vector<int> ri;      // [ntarget+1]
  std::vector<int> src;     // source index (mm index for M2D, pol index for D2D)
  std::vector<double> sP;   // scale for the P field (or the only field)
  std::vector<double> sD;   // scale for the D field (AMOEBA M2D only)
};

// Parse a revision 2/3 .mmp file (src/mod_inputloader.F90:15-257).
bool read_mmp(const std::string &path, HostModel &m, std::string &err);
// mmpol_prepare restated (src/mod_mmpol.F90:139-237), minus FMM.
bool prepare_model(HostModel &m, std::string &err);
// rotate_multipoles (src/rotate_multipoles.F90:232-295).
bool rotate_multipoles(HostModel &m, std::string &err);
// Target-major scaled-pair lists equivalent to make_screening_lists
// (src/mod_electrostatics.F90:538-864) and screening_rules (:3338-3487).
void build_m2d_pairs(const HostModel &m, ScaledPairs &out);
void build_d2d_pairs(const HostModel &m, ScaledPairs &out);

// Block-Jacobi preconditioner of the FP32 inner solver (precond.cpp): runs of
// at most kMaxBlock consecutive polarizable sites, each within kBlockLinkBohr
// of an earlier site of its run; per site {run start, run size, offset of the
// run's inverse block in minv, index in the run}; minv holds the FP32
// inverse of each run's diagonal block of T, (3 size) x (3 size) row-major.
constexpr int kMaxBlock = 8;
constexpr double kBlockLinkBohr = 3.0;
constexpr int kMaxBlockLimit = 32;
void build_block_jacobi(const HostModel &m, const ScaledPairs &d2d, double damp_thr, int max_sites,
                        double link_bohr, std::vector<int> &info, std::vector<float> &minv);
// Near-field couplings of the inner preconditioner's Neumann step: for each
// polarizable site j (row), the sites i of other runs (info from
// build_block_jacobi) within rc, with the 3x3 block of T between them,
// -s (3 k5 d d^T - k3 I) with the damping and the D2D scale of the product
// (row-major, FP32): CSR ri [n + 1], ci [nnz], blk [nnz][9]
constexpr double kNearBohr = 6.5;
void build_near_field(const HostModel &m, const ScaledPairs &d2d, double damp_thr, const std::vector<int> &info,
                      double rc, std::vector<int> &ri, std::vector<int> &ci, std::vector<float> &blk);

}  // namespace ommp
