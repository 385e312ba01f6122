// afg_transport.cuh -- drift-diffusion transport state (filled in below).
#pragma once
namespace afg {
struct TransportState {};
inline void transport_free(TransportState&) {}
}  // namespace afg
