// FLOP-count build of the oracle only (make opcount) -- TEST INFRASTRUCTURE
// ONLY.  Reads and clears the calling thread's operation counters of
// opcount.hpp; run the counted calls with one thread.
extern "C" {

void orc_opcount_reset() {
  for (int k = 0; k < opc::NKIND; ++k) opc::g_count[k] = 0;
}

void orc_opcount_get(unsigned long long* out) {
  for (int k = 0; k < opc::NKIND; ++k) out[k] = opc::g_count[k];
}

}  // extern "C"
