# Package root: csrc/ (CUDA kernels + C ABI), mushy_gb300/ (Python host mirror).
