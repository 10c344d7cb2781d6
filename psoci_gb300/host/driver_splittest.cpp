// psoci_driver: the production flow of the reference driver (driver.PSOCI.splittest.C:280-1511)
// on one GPU through the C++ host mirror (include/psoci/PsociGpu.hpp) and the C ABI.
//
//   configurations -> determinants -> H (or H restart) -> Davidson -> eigenvalues, vectors
//
// Flags follow the reference's getopt letters (driver.PSOCI.splittest.C:80-265) where the
// meaning carries over:
//   -c configs file   -m integral file (PSOCIINT binary, stands in for the SIFS moints file)
//   -n roots          -F final residual tolerance      -x subspace max multiplier
//   -I max iterations -v vector file (ASCII PsociVector layout)   -r restart from -v
//   -H read H checkpoint (-k path)   -W write H checkpoint (-k path)
// and for the GPU path:
//   -p 0|1  sigma precision (0 FP64, 1 mixed FP32/FP64 with FP64 refinement; default 1)
//   -b 0|1  block Davidson (default 1) or one vector per iteration as the reference
//   -d N    CUDA device
//   -L      the reference's own Davidson loop (driver.PSOCI.splittest.C:1186-1311: one new
//           vector per iteration for the first unconverged root, coarse 1e-3 then -F,
//           collapse to 2 x roots when the basis outgrows -x x roots) through the
//           step-level PsociGAbasis / PsociGAsubspace methods, FP64 products; without -L
//           the whole solve is one psoci_davidson call
//   -N      natural-orbital occupations of each root from its 1-particle density (the
//           reference's PsociNOpopulations step, driver.PSOCI.splittest.C:1420-1450; the
//           integral file carries no orbital symmetries, so all orbitals form one block)
// Output lines keep the reference's format (driver.PSOCI.splittest.C:1373):
//   "Eigenvalue i Total energy (au) E+core Electronic (au) E rnorm r"
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "psoci/PsociGpu.hpp"

// The reference's Davidson loop (driver.PSOCI.splittest.C:1050-1311 with INCREMENTAL,
// NEWRNOMRS, DIAGGOP and MODIFIED_EXPAND, the production flags) over the step-level mirror.
static psoci::PsociGAsubspace::Result referenceLoop(psoci::Device &dev, int64_t nsef, int numSoughtRoots, int maxmult,
                                                    int maxIterationsPerRtol, double rtol, bool restart) {
  const int minvecs = 2;
  const int maxsubspace = std::min<int64_t>(maxmult * numSoughtRoots, std::min<int64_t>(95, nsef - 1));
  psoci::PsociGAbasis vector_set(dev, numSoughtRoots, maxsubspace + 1);
  vector_set.setProducts(PSOCI_PREC_FP64);
  vector_set.specifyDiagonalGuessVectors(restart ? 2 : 0);
  vector_set.normAllVectors();
  if (int dep = vector_set.orthonormalizeAllVectors())
    throw psoci::Error(PSOCI_ERR_NUMERIC, "linear dependency in the guess vectors at " + std::to_string(dep));
  vector_set.computeHvProducts(0, numSoughtRoots);
  psoci::PsociGAsubspace subspace(dev, vector_set);
  std::vector<double> evals(maxsubspace + 1), rnorms(numSoughtRoots, -1.0);
  bool converged = false;
  int count = 0, total_count = 0, curroot = 1, compressSubspace = 0;
  int matrixVectorProducts = vector_set.CurrentExistingRoots();
  const double coarse_rtol = 0.001;
  double current_rtol = coarse_rtol;
  double rnormvalue = 0.0;
  int numUpdates = vector_set.CurrentExistingRoots();
  while (count < maxIterationsPerRtol && converged != true) {
    ++total_count;
    ++count;
    subspace.generateIncrementalSubspace(numUpdates);
    subspace.diagSubspaceGOP();
    subspace.brdcstEvals(evals);
    converged = true;
    int itest = curroot;
    while (itest <= numSoughtRoots) {
      subspace.computeRnormSingle(itest, evals, rnormvalue);
      rnorms[itest - 1] = rnormvalue;
      if (rnormvalue > current_rtol) {
        converged = false;
        curroot = itest;
        break;
      }
      ++itest;
    }
    if (converged == false) {
      double shift = evals[curroot - 1];
      vector_set.preconditionAndNewVectorIncore(curroot, shift);
      vector_set.appendScratchVector();
      matrixVectorProducts += 1;
      numUpdates = 1;
    }
    if (converged == true && current_rtol == coarse_rtol) {
      converged = false;
      count = 0;
      current_rtol = rtol;
      curroot = 1;
      if (vector_set.CurrentExistingRoots() >= minvecs * numSoughtRoots) {
        vector_set.expandAndReplaceVectorsNew(minvecs * numSoughtRoots);
        ++compressSubspace;
      }
      numUpdates = vector_set.CurrentExistingRoots();
    }
    if (vector_set.CurrentExistingRoots() > maxsubspace) {
      vector_set.expandAndReplaceVectorsNew(minvecs * numSoughtRoots);
      ++compressSubspace;
      numUpdates = vector_set.CurrentExistingRoots();
    }
  }
  subspace.computeRnorms(evals, rnorms);
  vector_set.expandAndReplaceVectorsNew(vector_set.CurrentExistingRoots());
  psoci::PsociGAsubspace::Result r;
  r.evals.assign(evals.begin(), evals.begin() + numSoughtRoots);
  r.rnorms = rnorms;
  r.evecs = vector_set.fetchVectors(numSoughtRoots, nsef);
  r.stats.iterations = total_count;
  r.stats.sigma_calls = matrixVectorProducts;
  r.stats.collapses = compressSubspace;
  if (!converged) throw psoci::Error(PSOCI_ERR_NOT_CONVERGED, "reference loop: not converged");
  return r;
}

int main(int argc, char **argv) {
  std::string cfg = "configs", moints = "moints", vecfile = "psoci_vectors.txt", hfile = "psoci_hamiltonian.bin";
  int nroots = 1, maxmult = 4, maxiter = 1000, prec = 1, block = 1, device = 0, verbose = 0;
  double rtol = 1e-6;
  bool restart = false, hread = false, hwrite = false, natorb = false, refloop = false;
  int c;
  while ((c = getopt(argc, argv, "c:m:n:F:x:I:v:rHWk:p:b:d:VNL")) != -1) {
    switch (c) {
      case 'c': cfg = optarg; break;
      case 'm': moints = optarg; break;
      case 'n': nroots = atoi(optarg); break;
      case 'F': rtol = atof(optarg); break;
      case 'x': maxmult = atoi(optarg); break;
      case 'I': maxiter = atoi(optarg); break;
      case 'v': vecfile = optarg; break;
      case 'r': restart = true; break;
      case 'H': hread = true; break;
      case 'W': hwrite = true; break;
      case 'k': hfile = optarg; break;
      case 'p': prec = atoi(optarg); break;
      case 'b': block = atoi(optarg); break;
      case 'd': device = atoi(optarg); break;
      case 'V': verbose = 1; break;
      case 'N': natorb = true; break;
      case 'L': refloop = true; break;
      default:
        std::cerr << "usage: psoci_driver -c configs -m ints [-n roots] [-F rtol] [-p 0|1] ..." << std::endl;
        return 2;
    }
  }
  try {
    auto t0 = std::chrono::steady_clock::now();
    psoci::PsociConfigs configs;
    configs.readConfigs(cfg);
    psoci::PsociIntegrals ints = psoci::PsociIntegrals::readFile(moints);
    psoci::Device dev(device, verbose);
    psoci::PsociGAhamiltonian ham(dev, ints);
    psoci::PsociGADeterminants dets(dev, configs);
    dets.generateDistributedDeterminantsSmallMemoryGA();
    const int64_t nsef = dets.fetchGlobalNumSefs();
    std::cout << "Number of configurations " << configs.numTotalSpatials() << " SEFs " << nsef << std::endl;
    psoci::PsociConstructHamiltonian store(dev);
    auto th = std::chrono::steady_clock::now();
    if (hread) {
      store.FetchHamiltonianFromDRA(hfile);
      std::cout << "Hamiltonian read from " << hfile << std::endl;
    } else {
      int64_t nnz = ham.constructGlobalHamiltonianAltOrbMapDirectChunkJmap(prec == 1);
      std::cout << "Hamiltonian non-zero elements " << nnz << std::endl;
    }
    double hsec = std::chrono::duration<double>(std::chrono::steady_clock::now() - th).count();
    if (hwrite) store.SendHamiltonianToDRA(hfile);

    psoci::PsociGAsubspace sub(dev);
    if (restart) {
      std::vector<double> guess;
      int k = psoci::PsociVector::read(vecfile, guess, nsef, nroots, false);
      sub.setGuess(k, guess);
      std::cout << "Restarted from " << k << " vectors in " << vecfile << std::endl;
    }
    psoci_dav_opts o{};
    o.nroots = nroots;
    o.max_subspace = maxmult * nroots;
    o.max_iter = maxiter;
    o.rtol = rtol;
    o.prec = prec == 1 ? PSOCI_PREC_MIXED : PSOCI_PREC_FP64;
    o.refine = 1;
    o.block = block;
    o.precond_min = 1e-3;
    psoci::PsociGAsubspace::Result r = refloop ? referenceLoop(dev, nsef, nroots, maxmult, maxiter, rtol, restart)
                                               : sub.solve(o, nsef, true);
    psoci::PsociVector::write(vecfile, r.evecs, nsef, nroots, false, "psoci_driver");
    double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const double fcore = ints.fetchCoreEnergy();
    std::cout << "Hamiltonian construction time " << hsec << std::endl;
    std::cout << "Number of SUBSPACE contractions is " << r.stats.collapses << std::endl;
    std::cout << "Number of total iterations is " << r.stats.iterations << std::endl;
    std::cout << "TOTAL MATRIX VECTOR PRODUCTS is " << r.stats.sigma_calls << std::endl;
    std::cout << "Current results: fcore is " << fcore << " " << std::endl;
    for (int i = 0; i < nroots; ++i)
      std::cout << "Eigenvalue " << i << " Total energy (au) " << std::setprecision(6) << r.evals[i] + fcore
                << " Electronic (au) " << std::setprecision(15) << r.evals[i] << " rnorm " << std::setprecision(10)
                << r.rnorms[i] << std::endl;
    if (natorb) {
      const int nbf = ints.nbf();
      std::vector<std::vector<double> > density;
      ham.constructCIdensityAltOrbMapChunkJmap(nroots, r.evecs, nbf, density);
      std::vector<int32_t> oneBlock(nbf, 1);
      for (int i = 0; i < nroots; ++i) {
        psoci::PsociNOpopulations::Root no = psoci::PsociNOpopulations::constructNaturalOrbitals(nbf, density[i], oneBlock);
        std::cout << "NO occupations root " << i << std::setprecision(8);
        for (int k = 0; k < nbf && k < 10; ++k) std::cout << " " << no.occupations[k];
        std::cout << std::endl;
      }
    }
    std::cout << "Total time (s) " << total << std::endl;
  } catch (const psoci::Error &e) {
    std::cerr << "psoci_driver: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}
