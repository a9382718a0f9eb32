// Runs a deck exported by `python -m fiesta_gb300.deck <deck.lua> <prefix>`
// through the C++ module interface: <prefix>.cfg, <prefix>.U0 (and .X for
// generalized grids, .noise when the deck enables the noise filter) in,
// <prefix>.U1 out after the given number of steps.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "fst_module.hpp"

int main(int argc, char** argv) {
  if (argc != 3) {
    std::printf("usage: module_deck <prefix> <steps>\n");
    return 2;
  }
  const std::string pre = argv[1];
  const int steps = std::atoi(argv[2]);
  try {
    const fst_config cf = fst::load_config(pre + ".cfg");
    auto f = fst::make_module(cf);
    fst_noise_params np;
    if (fst::load_noise(pre + ".noise", np)) f->set_noise(np);
    fst::load_array(pre + ".U0", f->var);
    if (auto* g = dynamic_cast<fst::gen_func*>(f.get())) fst::load_array(pre + ".X", g->grid);
    f->upload();
    f->preSim();
    for (int t = 0; t < steps; ++t) {
      f->preStep();
      fst::rkAdvance(*f);
      f->postStep();
    }
    f->postSim();
    f->download();
    FILE* o = std::fopen((pre + ".U1").c_str(), "wb");
    if (!o || std::fwrite(f->var.data(), sizeof(double), f->var.size(), o) != f->var.size())
      throw fst::Error(FST_ERR_INVALID, "write " + pre + ".U1");
    std::fclose(o);
  } catch (const fst::Error& e) {
    std::printf("fst::Error %d: %s\n", e.code, e.what());
    return 1;
  }
  std::printf("module_deck: ok\n");
  return 0;
}
