// QM helper object (qm_helper.cu): nuclei of a QM region and the
// electrostatic quantities between them and one polarizable system.
#pragma once

#include <vector>

namespace ommp {

class System;

class QMHelper {
 public:
  QMHelper(int n, const double *cqm, const double *qqm, const int *zqm);
  ~QMHelper();
  void update_coord(const double *cqm);
  int prepare_ene(System &s);
  int prepare_grd(System &s);

  int qm_atoms() const { return nq_; }
  double *cqm() { return cqm_.data(); }
  // [n][k] host arrays, or nullptr before they are computed
  double *E_n2p() { return e_n2p_done_ ? e_n2p_.data() : nullptr; }
  double *G_n2p() { return g_n2p_done_ ? g_n2p_.data() : nullptr; }
  double *E_n2m() { return e_n2m_done_ ? e_n2m_.data() : nullptr; }
  double *G_n2m() { return g_n2m_done_ ? g_n2m_.data() : nullptr; }
  double *H_n2m() { return h_n2m_done_ ? h_n2m_.data() : nullptr; }
  double *V_m2n() { return v_m2n_done_ ? v_m2n_.data() : nullptr; }
  double *V_p2n() { return v_p2n_done_ ? v_p2n_.data() : nullptr; }
  double *E_m2n() { return e_m2n_done_ ? e_m2n_.data() : nullptr; }
  double *E_p2n() { return e_p2n_done_ ? e_p2n_.data() : nullptr; }
  int npol() const { return e_n2p_done_ ? (int)(e_n2p_.size() / 3) : 0; }
  int nmm() const { return e_n2m_done_ ? (int)(e_n2m_.size() / 3) : 0; }

 private:
  int nuclear_fields(System &s, bool grad);
  int nq_;
  std::vector<double> cqm_, qqm_;
  std::vector<int> zqm_;
  std::vector<double> e_n2p_, g_n2p_, e_n2m_, g_n2m_, h_n2m_, v_m2n_, v_p2n_, e_m2n_, e_p2n_;
  bool e_n2p_done_ = false, g_n2p_done_ = false, e_n2m_done_ = false, g_n2m_done_ = false, h_n2m_done_ = false;
  bool v_m2n_done_ = false, v_p2n_done_ = false, e_m2n_done_ = false, e_p2n_done_ = false;
  double *dbuf_ = nullptr;  // device: nuclei and outputs
  size_t cap_ = 0;
};

}  // namespace ommp
