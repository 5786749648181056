"""Run the reference's own CUDA kernels (compiled by oracle/build_ref_gpu.py).

TEST INFRASTRUCTURE ONLY: used to generate the golden vectors under
tests/golden/.  Launch geometry and buffer layouts follow the reference host
code (GPUTileProcessor.java: setTasks 363-371, setConvolutionKernels 381-435,
setBayerImage 437-450, execConverCorrectTiles 530-558, execImcltRbg 560-597).
Device memory comes from torch; the cubin is loaded into torch's (primary)
context through the CUDA driver API.
"""
import ctypes as C

import numpy as np


class RefGpu:
    def __init__(self, cubin, width, height, num_cams=4, num_colors=3):
        import torch
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.cu = C.CDLL("libcuda.so.1")
        self._ck(self.cu.cuInit(0), "cuInit")
        data = open(cubin, "rb").read()
        self._image = C.create_string_buffer(data, len(data))
        self.mod = C.c_void_p()
        self._ck(self.cu.cuModuleLoadData(C.byref(self.mod), self._image), "cuModuleLoadData")
        self.f_cc = C.c_void_p()
        self.f_im = C.c_void_p()
        self._ck(self.cu.cuModuleGetFunction(C.byref(self.f_cc), self.mod, b"convert_correct_tiles"), "getfn")
        self._ck(self.cu.cuModuleGetFunction(C.byref(self.f_im), self.mod, b"imclt_rbg"), "getfn")
        self.W, self.H, self.NC, self.NCOL = width, height, num_cams, num_colors
        self.tilesX, self.tilesY = width // 8, height // 8
        self.KH, self.KV = width // 16 + 2, height // 16 + 2

    def _ck(self, r, what):
        if r != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, r))

    def get_global(self, name, count):
        """a float32 __constant__ / __device__ array of the module (e.g. lpf_data [3][64])"""
        ptr = C.c_uint64()
        size = C.c_size_t()
        self._ck(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, name.encode()), "getglobal")
        out = np.zeros(count, np.float32)
        self._ck(self.cu.cuMemcpyDtoH_v2(out.ctypes.data_as(C.c_void_p), ptr, C.c_size_t(count * 4)), "dtoh")
        return out

    def dtt24(self, img, mode):
        """GPU_DTT24_DRV (dtt8x8.cuh:100-158) on a float image whose width is a multiple of 32 and
        height of 16 (the kernel's 32x16-pixel blocks of 8x4x2 threads)"""
        torch = self.torch
        fn = C.c_void_p()
        self._ck(self.cu.cuModuleGetFunction(C.byref(fn), self.mod, b"GPU_DTT24_DRV"), "getfn")
        h, w = img.shape
        src = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32)).to("cuda")
        dst = torch.zeros_like(src)
        torch.cuda.synchronize()
        self._launch(fn, (w // 32, h // 16, 1), (8, 4, 2),
                     [C.c_uint64(dst.data_ptr()), C.c_uint64(src.data_ptr()), C.c_int(w), C.c_int(mode)])
        self._ck(self.cu.cuCtxSynchronize(), "sync")
        return dst.cpu().numpy()

    def _launch(self, fn, grid, block, args):
        holders = []
        ptrs = (C.c_void_p * len(args))()
        for i, a in enumerate(args):
            holders.append(a)
            ptrs[i] = C.cast(C.pointer(a), C.c_void_p)
        self._ck(self.cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0, None, ptrs,
                                        None), "cuLaunchKernel")

    def run(self, mosaics, kernels_gpu, offsets, tasks_packed, lpf_mask=0):
        """mosaics [4][H][W] f32; kernels_gpu [4][kv][kh][3][4][64] (transposed upload layout);
        offsets [4][kv][kh][3][8]; tasks_packed [n][10] TpTask floats.
        Returns clt [4][tilesY][tilesX][3][4][64] and rbg [4][3][H+8][W+8]."""
        torch = self.torch
        dev = "cuda"
        pitch = self.W  # dense pitch (the reference uses cuMemAllocPitch; any pitch >= width is valid)
        imgs = [torch.from_numpy(np.ascontiguousarray(m, dtype=np.float32)).to(dev) for m in mosaics]
        kers = [torch.from_numpy(np.ascontiguousarray(k, dtype=np.float32)).to(dev) for k in kernels_gpu]
        offs = [torch.from_numpy(np.ascontiguousarray(o, dtype=np.float32)).to(dev) for o in offsets]
        clts = [torch.zeros((self.tilesY, self.tilesX, self.NCOL, 256), dtype=torch.float32, device=dev)
                for _ in range(self.NC)]
        istride = self.W + 8
        rbgs = [torch.zeros((self.NCOL * (self.H + 8), istride), dtype=torch.float32, device=dev)
                for _ in range(self.NC)]
        ptr = lambda ts: torch.tensor([t.data_ptr() for t in ts], dtype=torch.int64, device=dev)
        p_k, p_o, p_i, p_c = ptr(kers), ptr(offs), ptr(imgs), ptr(clts)
        tasks = torch.from_numpy(np.ascontiguousarray(tasks_packed, dtype=np.float32)).to(dev)
        n = tasks_packed.shape[0]
        torch.cuda.synchronize()
        self._launch(self.f_cc, ((n + 3) // 4, 1, 1), (8, 4, 1),
                     [C.c_uint64(p_o.data_ptr()), C.c_uint64(p_k.data_ptr()), C.c_uint64(p_i.data_ptr()),
                      C.c_uint64(tasks.data_ptr()), C.c_uint64(p_c.data_ptr()), C.c_size_t(pitch), C.c_int(n),
                      C.c_int(lpf_mask)])
        self._ck(self.cu.cuCtxSynchronize(), "sync")
        for cam in range(self.NC):
            for color in range(self.NCOL):
                for v in range(2):
                    for h in range(2):
                        ty_half = (self.tilesY + (v ^ 1)) >> 1
                        tx_half = (self.tilesX + (h ^ 1)) >> 1
                        nt = ty_half * tx_half
                        self._launch(self.f_im, ((nt + 3) // 4, 1, 1), (16, 4, 1),
                                     [C.c_uint64(clts[cam].data_ptr()), C.c_uint64(rbgs[cam].data_ptr()),
                                      C.c_int(color), C.c_int(v), C.c_int(h), C.c_size_t(istride)])
                        self._ck(self.cu.cuCtxSynchronize(), "sync")
        clt = np.stack([c.cpu().numpy().reshape(self.tilesY, self.tilesX, self.NCOL, 4, 64) for c in clts])
        rbg = np.stack([r.cpu().numpy().reshape(self.NCOL, self.H + 8, istride) for r in rbgs])
        return clt, rbg
