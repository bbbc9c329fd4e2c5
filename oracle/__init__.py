"""CPU oracle (test infrastructure only): a restatement of the fhe.rs RNS-BFV
hot path used to check the GPU library bit for bit. Never imported by the
GPU product."""
