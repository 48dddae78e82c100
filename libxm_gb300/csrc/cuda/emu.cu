/* placeholder until the split-precision path lands */
#include <vector>
#include "common.cuh"
namespace xmg {
int emu_contract(xmgd_contract_t *, const std::vector<int> &,
    const xmgd_cblock_t *, const xmgd_pair_t *, const int32_t *,
    xmgd_timing_t *)
{
	return xmg_seterr(XMG_ENOTSUP, "split-precision path not built");
}
}
