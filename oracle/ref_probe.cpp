// Probe driver that calls the reference's own hot-path functions directly and
// prints their results as C99 hex floats, one value per token.  Test
// infrastructure only: it is compiled against the reference sources by
// `make -C oracle ref` and used by tests/golden/make_golden.py to generate the
// committed golden vectors.  Nothing in the product links it.
//
// Commands (all options come from a reference params file, parsed by the
// reference's own optionParser, src/optionsParser.cpp:177):
//   ref_probe init   PARAMS          initParticlesCPU (src/particle.cpp:638) for
//                                     numParticles particles; prints per particle
//                                     pos, v, next_gas_coll_time, rng x y z w
//   ref_probe draws  PARAMS K        per particle after init: K raw xoshiro
//                                     outputs (src/particle.cpp:59), then K
//                                     normal(0,1) draws (src/particle.cpp:89)
//   ref_probe dop    PARAMS t0 tf y0x y0y y0z px py pz vx vy vz h
//   ref_probe rk45   PARAMS ...same...  integrateDOP / integrateRK45
//                                     (src/integrator.cpp:90, :251) over one
//                                     ballistic segment from (p, v) at t0;
//                                     prints ret, y, h
//   ref_probe magnus|rk45q|rkf45|rkf45q PARAMS ...same...
//                                     integrateMagnusCFET (:625),
//                                     integrateRK45Quaternion (:441),
//                                     integrateRKF45 (:339),
//                                     integrateRKF45Quaternion (:530) likewise
//   ref_probe options PARAMS         the options image optionParser produced
//                                     (src/optionsParser.cpp:177), derived as
//                                     mainAnalysis does, as hex bytes
//   ref_probe events PARAMS NSEG      per particle after init: NSEG rounds of
//                                     calc_next_collision_time + update +
//                                     sanity_check (src/particle.cpp:121-444)
//                                     with tf = opt.tf; prints per segment
//                                     coll_type wall_hit dt t pos v next_gas
//   ref_probe sizes PARAMS            sizeof options, coords, rngState,
//                                     SpectrumAggregator, floquetDiagonalization
//   ref_probe spectrum PARAMS ax ay az wx wy wz
//                                     integratorType 6 (noise amplitudes a and
//                                     frequencies w set, the params file has no
//                                     keys for them): floquet_diagonalize
//                                     (src/integrator.cpp:824) frequencies and
//                                     dt, then per particle the first window of
//                                     runSimulationCPU's loop (src/particle.cpp:
//                                     746-800) with integrateSpectrum, and the
//                                     aggregator's state at its end: samples,
//                                     bounces, collisions, s1, s2, imag_diag
#include "include/particle.h"
#include "include/optionsParser.h"
#include "include/integrator.h"
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cstring>

static void hx(double x) { std::printf(" %a", x); }

static options load(const char* path) {
  options opt = optionParser(const_cast<char*>(path));
  const double k = 1.380649e-23;  // same derivation as src/simulation.cpp:9-11
  opt.tc = 1.6e-4 * opt.m / (k * pow(opt.T, 8.0));
  opt.sqrtKT_m = sqrt(k * opt.T / opt.m);
  return opt;
}

struct Arrays {
  int n;
  std::vector<coords> S, v, v_old, pos, pos_old;
  std::vector<double> t, t_old, tf, dt, next_gas, h;
  std::vector<rngState> state;
  std::vector<size_t> n_bounce, n_coll, n_steps;
  std::vector<unsigned int> partID;
  std::vector<int> fail;
  std::vector<bool> stop_unused;
  bool* stop;
  std::vector<char> coll_type, wall_hit;
  SpectrumAggregator* spec;
  explicit Arrays(int n_) : n(n_), S(n), v(n), v_old(n), pos(n), pos_old(n), t(n), t_old(n), tf(n),
      dt(n), next_gas(n), h(n), state(n), n_bounce(n), n_coll(n), n_steps(n), partID(n), fail(n),
      coll_type(n), wall_hit(n) {
    stop = new bool[n];
    spec = new SpectrumAggregator[n];
  }
};

// SpectrumAggregator's members in their declaration order (include/floquet.h:
// 76-95), to read the private accumulators of an aggregator the reference ran.
struct SpecMirror {
  int n_samples;
  coords s1[NW];
  coords s2[NW];
  covMat cmat[NW];
  double w[NW];
  double dt;
};
static_assert(sizeof(SpecMirror) == sizeof(SpectrumAggregator), "SpectrumAggregator layout");

static void init_all(const options& opt, Arrays& a, floquetDiagonalization fd = floquetDiagonalization{}) {
  initParticlesCPU(opt, a.S.data(), a.v.data(), a.v_old.data(), a.pos.data(), a.pos_old.data(),
                   a.t.data(), a.t_old.data(), a.tf.data(), a.dt.data(), a.next_gas.data(), a.h.data(),
                   a.state.data(), a.n_bounce.data(), a.n_coll.data(), a.n_steps.data(), a.partID.data(),
                   a.fail.data(), a.stop, a.coll_type.data(), a.wall_hit.data(), a.spec, fd);
}

int main(int argc, char** argv) {
  if (argc < 3) { std::fprintf(stderr, "usage: ref_probe CMD PARAMS ...\n"); return 2; }
  const char* cmd = argv[1];
  options opt = load(argv[2]);
  if (!std::strcmp(cmd, "options")) {  // the parsed (and derived) options image, as hex bytes
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&opt);
    std::printf("options ");
    for (size_t k = 0; k < sizeof(opt); ++k) std::printf("%02x", b[k]);
    std::printf("\n");
    return 0;
  }
  if (!std::strcmp(cmd, "init") || !std::strcmp(cmd, "draws") || !std::strcmp(cmd, "events")) {
    Arrays a(opt.numParticles);
    init_all(opt, a);
    for (int i = 0; i < a.n; ++i) {
      std::printf("p %d", i);
      if (!std::strcmp(cmd, "init")) {
        hx(a.pos[i].x); hx(a.pos[i].y); hx(a.pos[i].z);
        hx(a.v[i].x); hx(a.v[i].y); hx(a.v[i].z);
        hx(a.next_gas[i]);
        std::printf(" %llu %llu %llu %llu %d", (unsigned long long)a.state[i].x, (unsigned long long)a.state[i].y,
                    (unsigned long long)a.state[i].z, (unsigned long long)a.state[i].w, (int)a.state[i].hasSpare);
        hx(a.state[i].hasSpare ? a.state[i].spare : 0.0);
        std::printf("\n");
      } else if (!std::strcmp(cmd, "draws")) {
        int k = std::atoi(argv[3]);
        rngState s = a.state[i];
        for (int j = 0; j < k; ++j) std::printf(" %llu", (unsigned long long)xoshiro256p(s));
        for (int j = 0; j < k; ++j) hx(normal(s, 0.0, 1.0));
        std::printf("\n");
      } else {
        int nseg = std::atoi(argv[3]);
        double t = a.t[i], t_old = a.t_old[i], ng = a.next_gas[i], dt = 0.0;
        coords pos = a.pos[i], pos_old = a.pos_old[i], v = a.v[i], v_old = a.v_old[i];
        rngState s = a.state[i];
        size_t nb = 0, nc = 0;
        char ct = 'W', wh = 0;
        bool fin = false, stop = false;
        int fail = 0;
        std::printf("\n");
        for (int j = 0; j < nseg && !fin && !stop; ++j) {
          calc_next_collision_time(t, opt.tf, v, pos, ng, dt, ct, nb, nc, fin, wh, s, opt);
          update_position_and_velocity(t_old, t, dt, pos_old, pos, v_old, v, ct, wh, s, stop, opt);
          sanity_check(t_old, t, pos_old, pos, v, v_old, ct, wh, stop, fail, opt);
          std::printf("s %c %c %d %d", ct, wh ? wh : '-', (int)stop, fail);
          hx(dt); hx(t); hx(pos.x); hx(pos.y); hx(pos.z); hx(v.x); hx(v.y); hx(v.z); hx(ng);
          std::printf(" %llu\n", (unsigned long long)s.x);
        }
      }
    }
    return 0;
  }
  if (!std::strcmp(cmd, "sizes")) {  // the struct sizes a launcher of the GPU kernels lays out
    std::printf("options %zu coords %zu rngState %zu SpectrumAggregator %zu floquetDiagonalization %zu\n",
                sizeof(options), sizeof(coords), sizeof(rngState), sizeof(SpectrumAggregator),
                sizeof(floquetDiagonalization));
    return 0;
  }
  if (!std::strcmp(cmd, "spectrum")) {
    if (argc < 9) { std::fprintf(stderr, "spectrum needs 6 numbers\n"); return 2; }
    opt.noiseAmplitudes = {std::strtod(argv[3], nullptr), std::strtod(argv[4], nullptr), std::strtod(argv[5], nullptr)};
    opt.noiseFrequencies = {std::strtod(argv[6], nullptr), std::strtod(argv[7], nullptr), std::strtod(argv[8], nullptr)};
    floquetDiagonalization fd = floquet_diagonalize(opt);
    std::printf("f");
    for (int k = 0; k < NW; ++k) hx(fd.frequencies[k]);
    hx(fd.dt);
    std::printf("\n");
    Arrays a(opt.numParticles);
    init_all(opt, a, fd);
    for (int i = 0; i < a.n; ++i) {
      SpectrumAggregator specagg = a.spec[i];
      specagg.reset();
      const double tf = opt.ioutInt;  // the first window
      double t = a.t[i], t_old = a.t_old[i], ng = a.next_gas[i], dt = 0.0, tempH = a.h[i];
      coords pos = a.pos[i], pos_old = a.pos_old[i], v = a.v[i], v_old = a.v_old[i];
      rngState st = a.state[i];
      size_t nb = 0, nc = 0;
      char ct = 'W', wh = 0;
      bool fin = false, stop = false;
      int fail = 0;
      while (!fin && !stop) {
        calc_next_collision_time(t, tf, v, pos, ng, dt, ct, nb, nc, fin, wh, st, opt);
        update_position_and_velocity(t_old, t, dt, pos_old, pos, v_old, v, ct, wh, st, stop, opt);
        sanity_check(t_old, t, pos_old, pos, v, v_old, ct, wh, stop, fail, opt);
        if (fail == 0) integrateSpectrum(t_old, t, specagg, pos_old, pos, v_old, v, opt, tempH);
      }
      SpecMirror m;
      std::memcpy(&m, &specagg, sizeof(m));
      std::printf("p %d %d %d %llu %llu", i, m.n_samples, fail, (unsigned long long)nb, (unsigned long long)nc);
      for (int k = 0; k < NW; ++k) { hx(m.s1[k].x); hx(m.s1[k].y); hx(m.s1[k].z); }
      for (int k = 0; k < NW; ++k) { hx(m.s2[k].x); hx(m.s2[k].y); hx(m.s2[k].z); }
      for (int k = 0; k < NW; ++k) { hx(m.cmat[k].imag_diag.x); hx(m.cmat[k].imag_diag.y); hx(m.cmat[k].imag_diag.z); }
      std::printf("\n");
    }
    return 0;
  }
  const bool stepper = !std::strcmp(cmd, "dop") || !std::strcmp(cmd, "rk45") || !std::strcmp(cmd, "magnus") ||
                       !std::strcmp(cmd, "rk45q") || !std::strcmp(cmd, "rkf45") || !std::strcmp(cmd, "rkf45q");
  if (stepper) {
    if (argc < 16) { std::fprintf(stderr, "%s needs 13 numbers\n", cmd); return 2; }
    double vals[13];
    for (int j = 0; j < 13; ++j) vals[j] = std::strtod(argv[3 + j], nullptr);
    double t0 = vals[0], tf = vals[1];
    coords y = {vals[2], vals[3], vals[4]};
    coords p = {vals[5], vals[6], vals[7]};
    coords v = {vals[8], vals[9], vals[10]};
    double h = vals[11];
    (void)vals[12];
    // end-of-segment state is only used by the reference for signature parity
    coords p_new = p, v_new = v;
    int ret;
    if (!std::strcmp(cmd, "dop")) ret = integrateDOP(t0, tf, y, p, p_new, v, v_new, opt, h);
    else if (!std::strcmp(cmd, "rk45")) ret = integrateRK45(t0, tf, y, p, p_new, v, v_new, opt, h);
    else if (!std::strcmp(cmd, "magnus")) ret = integrateMagnusCFET(t0, tf, y, p, p_new, v, v_new, opt, h);
    else if (!std::strcmp(cmd, "rk45q")) ret = integrateRK45Quaternion(t0, tf, y, p, p_new, v, v_new, opt, h);
    else if (!std::strcmp(cmd, "rkf45")) ret = integrateRKF45(t0, tf, y, p, p_new, v, v_new, opt, h);
    else ret = integrateRKF45Quaternion(t0, tf, y, p, p_new, v, v_new, opt, h);
    std::printf("r %d", ret);
    hx(y.x); hx(y.y); hx(y.z); hx(h);
    std::printf("\n");
    return 0;
  }
  std::fprintf(stderr, "unknown command %s\n", cmd);
  return 2;
}
