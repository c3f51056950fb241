// Drives the reference estimators' own main() functions (mi.cpp:15,
// transs.cpp:17, autoent.cpp:17, negs.cpp:15, kldiv.cpp:15, dens.cpp:109)
// through a stand-in variables_map. Input and output are the reference's
// ASCII files. Test infrastructure only.
#include <boost/program_options.hpp>

#include <string>

#include "autoent.hpp"
#include "dens.hpp"
#include "kldiv.hpp"
#include "mi.hpp"
#include "negs.hpp"
#include "transs.hpp"
#include "tools.hpp"

namespace po = boost::program_options;

extern "C" int ref_run_mode(const char* mode, const char* input,
                            const char* bandwidths, const char* output,
                            unsigned tau, unsigned dims, const char* taus) {
  po::variables_map a;
  a["input"] = po::variable_value::of(std::string(input));
  a["output"] = po::variable_value::of(std::string(output));
  a["columns"] = po::variable_value::of(std::string(""));
  a["bandwidths"] = po::variable_value::of(std::string(bandwidths));
  a["bits"] = po::variable_value::of(false);
  a["tau"] = po::variable_value::of(tau);
  a["dims"] = po::variable_value::of(dims);
  a["taus"] = po::variable_value::of(std::string(taus));
  std::string m(mode);
  if (m == "mi") Mi::main(a);
  else if (m == "transs") Transs::main(a);
  else if (m == "autoent") AutoEnt::main(a);
  else if (m == "negs") Negs::main(a);
  else if (m == "kldiv") KLDiv::main(a);
  else if (m == "dens") Dens::main(a);
  else return 1;
  Tools::IO::set_out("");
  return 0;
}
