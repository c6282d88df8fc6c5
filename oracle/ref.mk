# Builds the reference's own host code from its sources, where they lie, into
# oracle/_ref/libref_crypt.so (git-ignored).  Test infrastructure only: it is
# the checker that pins the C restatement (oracle/crypt_oracle.c) and the
# golden fixtures; it is never linked into the product.
#
#   make -f oracle/ref.mk REF=/root/reference
#
# Only the host-callable functions are used, so device code is compiled for a
# single architecture.  The reference's int128.h has no aarch64 host branch
# (int128.h:9-20), so this recipe is x86_64-only; on other hosts it reports
# that and stops.

REF ?= /root/reference
OUT := oracle/_ref
NVCC ?= nvcc
ECC := $(REF)/src/cuda-ecc-ed25519
SHA := $(REF)/src/cuda-sha256
ARCH := $(shell uname -m)

FLAGS := -O2 -gencode arch=compute_100,code=sm_100 -DENDIAN_NEUTRAL -DLTC_NO_ASM \
         -I$(ECC) -I$(SHA) -I$(REF)/src/common -Xcompiler -fPIC -w

all: $(OUT)/libref_crypt.so

ifeq ($(ARCH),x86_64)
$(OUT)/ref_ed25519.o: oracle/ref_unity.cu
	@mkdir -p $(OUT)
	$(NVCC) $(FLAGS) -c $< -o $@

$(OUT)/ref_sha256.o: oracle/ref_sha256_unity.cu
	@mkdir -p $(OUT)
	$(NVCC) $(FLAGS) -c $< -o $@

$(OUT)/libref_crypt.so: $(OUT)/ref_ed25519.o $(OUT)/ref_sha256.o
	$(NVCC) -shared -o $@ $^ -lcudart
else
$(OUT)/libref_crypt.so:
	@echo "oracle/_ref: reference host code needs x86_64 (int128.h); skipped on $(ARCH)"
endif

.PHONY: all
