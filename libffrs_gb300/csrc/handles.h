// Definitions of the opaque C-ABI handles, shared by the entry points of each
// codec and by the batch API.
#pragma once

#include <memory>
#include <mutex>

#include "circ16.cuh"
#include "common.cuh"
#include "rs256.cuh"
#include "rsi16.cuh"

struct ffgpu_rs256 {
    std::unique_ptr<ffgpu::Rs256Code> code;
    std::mutex mu;
    ffgpu::DeviceBuffer d_data, d_parity, d_status;
    ffgpu::PinnedBuffer h_data, h_parity, h_status;
};

struct ffgpu_rsi16 {
    std::unique_ptr<ffgpu::Rsi16Code> code;
    std::mutex mu;
    ffgpu::DeviceBuffer d_msg, d_par, d_status, d_pos;
    ffgpu::PinnedBuffer h_msg, h_par, h_status;
};

struct ffgpu_circ16 {
    std::unique_ptr<ffgpu::Circ16Code> code;
    std::mutex mu;
    ffgpu::DeviceBuffer d_msg, d_ecc, d_status;
};
