// Driver appended (by oracle/build_ref.sh) after the reference's packbits.cu in one translation
// unit, so that the reference's own pack_bits_kernel runs on the CPU.  TEST INFRASTRUCTURE ONLY.
extern "C" {
void ref_packbits(std::uint32_t n_bytes, const float *thr, const float *density, bool *mask,
                  std::uint8_t *bits) {
    run_grid((n_bytes + 511) / 512, 512, false,
             [&]() { volrendjax::pack_bits_kernel(n_bytes, thr, density, mask, bits); });
}
}
