// C++ host mirror of the reference's Hamiltonian-build / Davidson path over the C ABI of
// libpsoci_gpu.so.  Header-only; include this one header.
//
// The classes keep the names and the main method names of the reference interfaces they
// replace (PsociIntegrals, PsociConfigs, PsociHamiltonian, PsociGAhamiltonian,
// PsociConstructHamiltonian, PsociGAsubspace, PsociVector — paths inside psociRestart-Cori/),
// inside namespace psoci so they can sit beside the reference's own classes.  The one
// unavoidable change is that Global Arrays handles become a psoci::Device (one GPU, one
// stream) owning the device arrays.  Errors throw psoci::Error carrying the C status.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../psoci_gpu.h"

namespace psoci {

class Error : public std::runtime_error {
 public:
  Error(psoci_status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
  psoci_status status;
};

inline void check(const psoci_ctx *c, psoci_status s, const char *what) {
  if (s == PSOCI_OK) return;
  std::string m = std::string(what) + ": " + psoci_status_str(s);
  if (c) m += std::string(" (") + psoci_last_error(c) + ")";
  throw Error(s, m);
}

// One GPU context (replaces GA::Initialize and the GA arrays of the H and vector spaces).
class Device {
 public:
  explicit Device(int device = 0, int verbose = 0) {
    psoci_opts o{device, verbose};
    check(nullptr, psoci_create(&ctx_, &o), "psoci_create");
  }
  ~Device() { psoci_destroy(ctx_); }
  Device(const Device &) = delete;
  Device &operator=(const Device &) = delete;
  psoci_ctx *get() const { return ctx_; }

 private:
  psoci_ctx *ctx_ = nullptr;
};

// PsociIntegrals (PsociIntegrals.hpp): packed one-electron table with the spin-orbit values
// folded in (PsociIntegrals.C:505-535) and the canonical two-electron table (:889-909).
class PsociIntegrals {
 public:
  PsociIntegrals() = default;
  PsociIntegrals(int nbf, std::vector<double> one, std::vector<double> eri, double ecore)
      : nbf_(nbf), one_(std::move(one)), eri_(std::move(eri)), ecore_(ecore) {}

  // Binary integral file written by psoci_gb300.inputs.write_integral_file:
  // "PSOCIINT", int32 nbf, double ecore, one[nbf(nbf+1)/2], eri[NNDAF(NNDAF(nbf))].
  // Stands in for fetchAndProcessIntegrals (:914-961), which reads Columbus SIFS files.
  static PsociIntegrals readFile(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(PSOCI_ERR_IO, "cannot open integral file " + path);
    char magic[8];
    int32_t nbf = 0;
    double ecore = 0.0;
    f.read(magic, 8);
    f.read(reinterpret_cast<char *>(&nbf), 4);
    f.read(reinterpret_cast<char *>(&ecore), 8);
    if (!f || std::string(magic, 8) != "PSOCIINT" || nbf < 1 || nbf > 128)
      throw Error(PSOCI_ERR_IO, "bad integral file header " + path);
    int64_t n1 = (int64_t)nbf * (nbf + 1) / 2, n2 = n1 * (n1 + 1) / 2;
    std::vector<double> one(n1), eri(n2);
    f.read(reinterpret_cast<char *>(one.data()), 8 * n1);
    f.read(reinterpret_cast<char *>(eri.data()), 8 * n2);
    if (!f) throw Error(PSOCI_ERR_IO, "truncated integral file " + path);
    return PsociIntegrals(nbf, std::move(one), std::move(eri), ecore);
  }

  double fetch1eIntegralValue(int i, int j) const { return one_[tri(i, j)]; }
  double fetch2eIntegralValue(int i, int j, int k, int l) const { return eri_[tri(tri(i, j), tri(k, l))]; }
  double fetchCoreEnergy() const { return ecore_; }
  int nbf() const { return nbf_; }
  const std::vector<double> &one() const { return one_; }
  const std::vector<double> &eri() const { return eri_; }

 private:
  static int64_t tri(int64_t i, int64_t j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }
  int nbf_ = 0;
  std::vector<double> one_, eri_;
  double ecore_ = 0.0;
};

// PsociConfigs (PsociConfigs.hpp): the configuration file — title; "nbf nelec ksym ncfgs
// nopen"; then "jsym occupation-string" lines (PsociConfigs.C:126-302).  The reference
// rejects configurations without a doubly occupied orbital (PsociConfigs.C:247);
// allowAllOpen (default) accepts them.
class PsociConfigs {
 public:
  int readConfigs(const std::string &path, bool allowAllOpen = true) {
    std::ifstream f(path);
    if (!f) throw Error(PSOCI_ERR_IO, "cannot open configuration file " + path);
    std::string line;
    std::getline(f, title_);
    if (!std::getline(f, line)) throw Error(PSOCI_ERR_IO, "configuration file too short");
    std::istringstream h(line);
    int ncfg = 0, nopen_hdr = 0;
    if (!(h >> nbf_ >> nelec_ >> ksym_ >> ncfg >> nopen_hdr)) throw Error(PSOCI_ERR_IO, "bad header line");
    jsym_.clear();
    occ_.clear();
    mx_open_ = 0;
    int js;
    std::string occ;
    while (f >> js >> occ) {
      if ((int)occ.size() != nbf_) throw Error(PSOCI_ERR_IO, "occupation string of the wrong length");
      int ne = 0, no = 0;
      for (char ch : occ) {
        if (ch < '0' || ch > '2') throw Error(PSOCI_ERR_IO, "occupation digit outside 0..2");
        ne += ch - '0';
        no += (ch == '1');
        occ_.push_back((uint8_t)(ch - '0'));
      }
      if (ne != nelec_) throw Error(PSOCI_ERR_IO, "configuration with the wrong electron count");
      if (!allowAllOpen && no == ne) throw Error(PSOCI_ERR_IO, "configuration without a doubly occupied orbital");
      if (no > mx_open_) mx_open_ = no;
      jsym_.push_back(js);
    }
    if ((int)jsym_.size() != ncfg) throw Error(PSOCI_ERR_IO, "configuration count differs from the header");
    return ncfg;
  }
  int fetchNumBasisFtns() const { return nbf_; }
  int fetchNumElectrons() const { return nelec_; }
  int fetchStateSymmetry() const { return ksym_; }
  int fetchMaxOpenShells() const { return mx_open_; }
  int numTotalSpatials() const { return (int)jsym_.size(); }
  const std::vector<int32_t> &jsym() const { return jsym_; }
  const std::vector<uint8_t> &occ() const { return occ_; }

 private:
  std::string title_;
  int nbf_ = 0, nelec_ = 0, ksym_ = 0, mx_open_ = 0;
  std::vector<int32_t> jsym_;
  std::vector<uint8_t> occ_;
};

// PsociGADeterminants / PsociDeterminants::computeConfigs: determinants on the device.
class PsociGADeterminants {
 public:
  PsociGADeterminants(Device &d, const PsociConfigs &cf) : dev_(d) {
    check(dev_.get(), psoci_set_configs(dev_.get(), cf.fetchNumBasisFtns(), cf.fetchNumElectrons(),
                                        cf.fetchStateSymmetry(), cf.fetchMaxOpenShells(), cf.numTotalSpatials(),
                                        cf.jsym().data(), cf.occ().data()),
          "psoci_set_configs");
  }
  // generateDistributedDeterminantsSmallMemoryGA (PsociGADeterminants.C:1608-1731)
  void generateDistributedDeterminantsSmallMemoryGA() {
    check(dev_.get(), psoci_build_determinants(dev_.get()), "psoci_build_determinants");
    check(dev_.get(), psoci_get_counts(dev_.get(), &nsef_, &ndet_, &maxsef_, &maxdet_), "psoci_get_counts");
  }
  int64_t fetchGlobalNumSefs() const { return nsef_; }
  int64_t fetchGlobalNumDets() const { return ndet_; }
  int fetchGlobalMaxSefPerSpatial() const { return maxsef_; }
  int fetchGlobalMaxDetPerSpatial() const { return maxdet_; }

 private:
  Device &dev_;
  int64_t nsef_ = 0, ndet_ = 0;
  int maxsef_ = 0, maxdet_ = 0;
};

// PsociHamiltonian (PsociHamiltonian.hpp): one configuration-pair block, reference roles.
class PsociHamiltonian {
 public:
  explicit PsociHamiltonian(Device &d) : dev_(d) {}
  // generateSOCIblocks(iconf, jconf, sefsef) (PsociHamiltonian.C:401-558); 0-based indices.
  void generateSOCIblocks(int iconf, int jconf, std::vector<double> &sefsef, int nsefi, int nsefj) {
    sefsef.assign((size_t)nsefi * nsefj, 0.0);
    int32_t a = iconf, b = jconf;
    check(dev_.get(), psoci_blocks(dev_.get(), 1, &a, &b, sefsef.data()), "psoci_blocks");
  }

 private:
  Device &dev_;
};

// PsociGAhamiltonian (PsociGAhamiltonian.hpp): the stored H, its diagonal and sigma.
class PsociGAhamiltonian {
 public:
  PsociGAhamiltonian(Device &d, const PsociIntegrals &ints) : dev_(d) {
    check(dev_.get(), psoci_set_integrals(dev_.get(), ints.nbf(), ints.one().data(), ints.eri().data(),
                                          ints.fetchCoreEnergy()),
          "psoci_set_integrals");
  }
  // constructGlobalHamiltonianAltOrbMapDirectChunkJmap (PsociGAhamiltonian.C:2530-2857)
  int64_t constructGlobalHamiltonianAltOrbMapDirectChunkJmap(bool withFP32Copy = true) {
    check(dev_.get(), psoci_build_hamiltonian(dev_.get(), withFP32Copy ? PSOCI_HMODE_CSR_BOTH : PSOCI_HMODE_CSR_FP64,
                                              &nnz_),
          "psoci_build_hamiltonian");
    return nnz_;
  }
  // the reference's DIRECTMATRIXPRODUCTS build (PsociGAhamiltonian.C:7549-7826): nothing
  // stored, every matrixVectorProducts call evaluates the elements again
  void constructGlobalHamiltonianDirect() {
    check(dev_.get(), psoci_build_hamiltonian(dev_.get(), PSOCI_HMODE_DIRECT, &nnz_), "psoci_build_hamiltonian");
  }
  int64_t numberNonzeroElements() const { return nnz_; }
  // the build's element evaluation in one launch (launches = 1: less memory, slower; the
  // same matrix) or the automatic choice (0); no reference counterpart
  void setEvalLaunches(int launches) {
    check(dev_.get(), psoci_set_eval_launches(dev_.get(), launches), "psoci_set_eval_launches");
  }
  // constructCIdensityAltOrbMapChunkJmap (PsociGAhamiltonian.C:11570-11760): density[root] is
  // the packed nbf(nbf+1)/2 spin-free 1-particle density of root-major vectors vecs (k x N)
  int64_t constructCIdensityAltOrbMapChunkJmap(int numRoots, const std::vector<double> &vecs, int nbf,
                                               std::vector<std::vector<double> > &density) {
    const size_t ntri = (size_t)nbf * (nbf + 1) / 2;
    std::vector<double> flat((size_t)numRoots * ntri);
    check(dev_.get(), psoci_density1(dev_.get(), numRoots, vecs.data(), flat.data()), "psoci_density1");
    density.assign(numRoots, std::vector<double>());
    for (int r = 0; r < numRoots; ++r) density[r].assign(flat.begin() + r * ntri, flat.begin() + (r + 1) * ntri);
    return (int64_t)numRoots * (int64_t)ntri;
  }
  // fetchDIAG_SEF (PsociGAhamiltonian.C:9014)
  void fetchDIAG_SEF(std::vector<double> &diag, int64_t nsef) {
    diag.resize(nsef);
    check(dev_.get(), psoci_get_diag(dev_.get(), diag.data()), "psoci_get_diag");
  }
  // matrixVectorProductsSplitChunkMultipleJchunks (PsociGAhamiltonian.C:6921-7270): k vectors,
  // x and y N x k row-major
  void matrixVectorProducts(int k, const std::vector<double> &x, std::vector<double> &y, psoci_prec prec) {
    y.resize(x.size());
    check(dev_.get(), psoci_sigma(dev_.get(), k, x.data(), y.data(), prec), "psoci_sigma");
  }

 private:
  Device &dev_;
  int64_t nnz_ = 0;
};

// PsociConstructHamiltonian (PsociConstructHamiltonian.hpp): H restart files; the DRA store
// of the reference becomes one checkpoint file.
class PsociConstructHamiltonian {
 public:
  explicit PsociConstructHamiltonian(Device &d) : dev_(d) {}
  void SendHamiltonianToDRA(const std::string &path) {
    check(dev_.get(), psoci_save_hamiltonian(dev_.get(), path.c_str()), "psoci_save_hamiltonian");
  }
  void FetchHamiltonianFromDRA(const std::string &path) {
    check(dev_.get(), psoci_load_hamiltonian(dev_.get(), path.c_str()), "psoci_load_hamiltonian");
  }

 private:
  Device &dev_;
};

// PsociGAbasis (PsociGAbasis.hpp): the Davidson vectors V and their products H*V, on the
// device.  The step-level methods keep the reference's names so that its driver loop
// (driver.PSOCI.splittest.C:1186-1311) carries over; the basis stays orthonormal.
class PsociGAbasis {
 public:
  // PsociGAbasis(numSoughtRoots, hamilton, g_v, g_Hv): room for maxVectors vectors
  PsociGAbasis(Device &d, int numSoughtRoots, int maxVectors) : dev_(d) {
    check(dev_.get(), psoci_basis_create(dev_.get(), numSoughtRoots, maxVectors), "psoci_basis_create");
  }
  ~PsociGAbasis() { psoci_basis_destroy(dev_.get()); }
  PsociGAbasis(const PsociGAbasis &) = delete;
  PsociGAbasis &operator=(const PsociGAbasis &) = delete;
  // PsociGAvectors::specifyDiagonalGuessVectors (PsociGAvectors.C:687-726); mode 0 the
  // reference's unit vectors on the first SEFs, 1 the lowest diagonal elements, 2 restart
  // vectors given to PsociGAsubspace::setGuess
  void specifyDiagonalGuessVectors(int mode = 0) {
    check(dev_.get(), psoci_basis_guess(dev_.get(), mode), "psoci_basis_guess");
  }
  // precision of the H*v products (the reference's are FP64)
  void setProducts(psoci_prec prec) { prec_ = prec; }
  // normAllVectors + orthonormalizeAllVectors (PsociGAbasis.C:1044, :1210): 0, or the 1-based
  // column found linearly dependent
  void normAllVectors() {}
  int orthonormalizeAllVectors() {
    int dep = 0;
    psoci_status s = psoci_basis_orthonormalize_all(dev_.get(), &dep);
    if (s == PSOCI_ERR_NUMERIC) return dep;
    check(dev_.get(), s, "psoci_basis_orthonormalize_all");
    return 0;
  }
  // computeHvProducts(start, num) (PsociGAbasis.C:1610)
  int computeHvProducts(int start, int num) {
    check(dev_.get(), psoci_basis_compute_hv(dev_.get(), start, num, prec_), "psoci_basis_compute_hv");
    return num;
  }
  void setpresent_matrixProducts(int) {}  // the device basis counts its products itself
  // preconditionAndNewVectorIncore(curroot, shift, g_rnorms, g_diag) (PsociGAbasis.C:1807-1919)
  int preconditionAndNewVectorIncore(int curroot, double shift, double precondMin = 1e-3) {
    check(dev_.get(), psoci_basis_precondition_new(dev_.get(), curroot, shift, precondMin),
          "psoci_basis_precondition_new");
    return 1;
  }
  // appendScratchVector (PsociGAbasis.C:362): orthonormalise, append, form its H*v
  int appendScratchVector() {
    int n = 0;
    check(dev_.get(), psoci_basis_append_scratch(dev_.get(), prec_, &n), "psoci_basis_append_scratch");
    return n;
  }
  // expandAndReplaceVectorsNew(g_evecs, num) (PsociGAbasis.C:483-583)
  int expandAndReplaceVectorsNew(int num) {
    check(dev_.get(), psoci_basis_expand_replace(dev_.get(), num), "psoci_basis_expand_replace");
    return num;
  }
  int CurrentExistingRoots() const { return info(0); }
  int CurrentNumSoughtRoots() const { return info(1); }
  int CurrentMaxRoots() const { return info(2); }
  int CurrentExistingHVProducts() const { return info(3); }
  // the first k vectors, root-major (after the last expandAndReplaceVectorsNew: the solution)
  std::vector<double> fetchVectors(int k, int64_t nsef) const {
    std::vector<double> v((size_t)k * nsef);
    check(dev_.get(), psoci_basis_vectors(dev_.get(), k, v.data()), "psoci_basis_vectors");
    return v;
  }
  Device &device() const { return dev_; }

 private:
  int info(int which) const {
    int e = 0, so = 0, mx = 0, pr = 0;
    check(dev_.get(), psoci_basis_info(dev_.get(), &e, &so, &mx, &pr), "psoci_basis_info");
    return which == 0 ? e : which == 1 ? so : which == 2 ? mx : pr;
  }
  Device &dev_;
  psoci_prec prec_ = PSOCI_PREC_FP64;
};

// PsociGAsubspace (PsociGAsubspace.hpp): the projected problem of a PsociGAbasis, and the
// whole Davidson solve in one call (solve(), the fast path: all unconverged roots per
// iteration, mixed precision with refinement).
class PsociGAsubspace {
 public:
  explicit PsociGAsubspace(Device &d) : dev_(d) {}
  PsociGAsubspace(Device &d, PsociGAbasis &basis) : dev_(d), basis_(&basis) { (void)basis_; }
  struct Result {
    std::vector<double> evals, rnorms, evecs;  // evecs root-major (root r at r*N)
    psoci_dav_stats stats{};
  };
  Result solve(const psoci_dav_opts &o, int64_t nsef, bool wantVectors) {
    Result r;
    r.evals.resize(o.nroots);
    r.rnorms.resize(o.nroots);
    if (wantVectors) r.evecs.resize((size_t)o.nroots * nsef);
    check(dev_.get(), psoci_davidson(dev_.get(), &o, r.evals.data(), wantVectors ? r.evecs.data() : nullptr,
                                     r.rnorms.data(), &r.stats),
          "psoci_davidson");
    return r;
  }
  // the reference's -r restart: vectors from a previous run seed the next solve
  void setGuess(int k, const std::vector<double> &vecs) {
    check(dev_.get(), psoci_set_guess(dev_.get(), k, vecs.data()), "psoci_set_guess");
  }
  // generateIncrementalSubspace(num) (PsociGAsubspace.C:273-366)
  void generateIncrementalSubspace(int num) {
    check(dev_.get(), psoci_subspace_generate_incremental(dev_.get(), num), "psoci_subspace_generate_incremental");
  }
  // diagSubspaceGOP (PsociGAsubspace.C:1088-1171); the eigenvalues stay for brdcstEvals
  void diagSubspaceGOP() {
    int e = 0;
    check(dev_.get(), psoci_basis_info(dev_.get(), &e, nullptr, nullptr, nullptr), "psoci_basis_info");
    evals_.assign(std::max(e, 1), 0.0);
    check(dev_.get(), psoci_subspace_diag(dev_.get(), evals_.data()), "psoci_subspace_diag");
  }
  // brdcstEvals(evals): the eigenvalues of the last diagSubspaceGOP (the front of evals)
  void brdcstEvals(std::vector<double> &evals) const {
    if (evals.size() < evals_.size()) evals.resize(evals_.size());
    std::copy(evals_.begin(), evals_.end(), evals.begin());
  }
  // computeRnormSingle(iroot, evals, rnorm) (PsociGAsubspace.C:874-1000), iroot 1-based
  int computeRnormSingle(int iroot, const std::vector<double> &, double &rnormvec) {
    check(dev_.get(), psoci_subspace_rnorm_single(dev_.get(), iroot, &rnormvec), "psoci_subspace_rnorm_single");
    return 0;
  }
  // computeRnorms(evals, rnorms) (PsociGAsubspace.C:775-872)
  int computeRnorms(const std::vector<double> &, std::vector<double> &rnorms) {
    int so = 0;
    check(dev_.get(), psoci_basis_info(dev_.get(), nullptr, &so, nullptr, nullptr), "psoci_basis_info");
    rnorms.resize(so);
    check(dev_.get(), psoci_subspace_rnorms(dev_.get(), rnorms.data()), "psoci_subspace_rnorms");
    return 0;
  }
  void destroySubspace() {}

 private:
  Device &dev_;
  PsociGAbasis *basis_ = nullptr;
  std::vector<double> evals_;
};

// PsociNOpopulations (PsociNOpopulations.hpp): natural orbitals of the CI densities in the MO
// basis.  The AO transformation, Mulliken analysis and NO files need the MO coefficient file
// and stay with the caller.
class PsociNOpopulations {
 public:
  struct Root {
    std::vector<double> occupations;  // per block, largest first; blocks in ascending label order
    std::vector<double> vectors;      // per block n_b x n_b, natural orbital i contiguous
    std::vector<int32_t> orbitals;    // the orbitals of the blocks, in output order
  };
  // constructNaturalOrbitals (PsociNOpopulations.C:569-669), MO-basis part, one root
  static Root constructNaturalOrbitals(int nbf, const std::vector<double> &density, const std::vector<int32_t> &orbSym) {
    Root r;
    r.occupations.resize(nbf);
    r.orbitals.resize(nbf);
    size_t nvec = 0;
    std::vector<int32_t> labels(orbSym);
    std::sort(labels.begin(), labels.end());
    for (size_t i = 0; i < labels.size();) {
      size_t j = i;
      while (j < labels.size() && labels[j] == labels[i]) ++j;
      nvec += (j - i) * (j - i);
      i = j;
    }
    r.vectors.resize(nvec);
    check(nullptr, psoci_natural_orbitals(nbf, density.data(), orbSym.data(), r.occupations.data(), r.vectors.data(),
                                          r.orbitals.data()),
          "psoci_natural_orbitals");
    return r;
  }
};

// PsociVector (PsociVector.hpp): CI vector files in the reference's scalable layout.
class PsociVector {
 public:
  static void write(const std::string &path, const std::vector<double> &vecs, int64_t nbasis, int nroots,
                    bool binary, const std::string &title = "") {
    check(nullptr, psoci_write_vectors(path.c_str(), binary, nbasis, nroots, vecs.data(), title.c_str()),
          "psoci_write_vectors");
  }
  static int read(const std::string &path, std::vector<double> &vecs, int64_t nbasis, int maxRoots, bool binary) {
    vecs.assign((size_t)maxRoots * nbasis, 0.0);
    int n = 0;
    check(nullptr, psoci_read_vectors(path.c_str(), binary, nbasis, maxRoots, vecs.data(), &n), "psoci_read_vectors");
    vecs.resize((size_t)n * nbasis);
    return n;
  }
};

}  // namespace psoci
