# Builds the reference OpenZL C core, from its own sources where they lie,
# into oracle/_ref/libozl_ref.so. This is the test oracle's ground truth:
# tests and fixture generators load it to pin the CPU restatement in
# oracle/ozl_oracle.c and to produce reference frames. It is never linked
# into the product.
#
#   make -f oracle/ref.mk -j8   (REF: $OZL_REFERENCE, else /root/reference)
#   make -f oracle/ref.mk -j8 OUT=oracle/_ref/native EXTRA=-march=native
#       (the same sources with the host's vector extensions, for the CPU
#       baseline's second variant)
#
# Recipe: every src/openzl/**/*.c except the zstd/lz4 bindings (their
# third-party libraries are not vendored), replaced by oracle/ref_stubs.c,
# compiled with the reference's default release flags (-O3 -DNDEBUG, no
# -march). The x86-64 Huffman assembly loop is added on x86-64 hosts only.
REF     ?= $(or $(OZL_REFERENCE),/root/reference)
OUT     ?= oracle/_ref
CC      ?= gcc
CFLAGS  := -std=gnu11 -O3 -DNDEBUG -fPIC -fvisibility=default $(EXTRA) \
           -I$(REF)/src -I$(REF)/include -I$(REF) -w
SRCS    := $(shell find $(REF)/src/openzl -name '*.c' \
             -not -path '*/codecs/zstd/*' -not -path '*/codecs/lz4/*' | sort)
OBJS    := $(patsubst $(REF)/src/%.c,$(OUT)/obj/%.o,$(SRCS)) $(OUT)/obj/ref_stubs.o
ARCH    := $(shell uname -m)
ifeq ($(ARCH),x86_64)
OBJS    += $(OUT)/obj/huf_decompress_amd64.o
endif

all: $(OUT)/libozl_ref.so $(OUT)/ref_driver.so

$(OUT)/obj/%.o: $(REF)/src/%.c
	@mkdir -p $(dir $@)
	@$(CC) $(CFLAGS) -c $< -o $@

$(OUT)/obj/ref_stubs.o: oracle/ref_stubs.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) -c $< -o $@

$(OUT)/obj/huf_decompress_amd64.o: $(REF)/src/openzl/fse/decompress/huf_decompress_amd64.S
	@mkdir -p $(dir $@)
	$(CC) -fPIC -I$(REF)/include -I$(REF)/src -c $< -o $@

$(OUT)/libozl_ref.so: $(OBJS)
	$(CC) -shared -o $@ $(OBJS) -lm

$(OUT)/ref_driver.so: oracle/ref_driver.c $(OUT)/libozl_ref.so
	$(CC) $(CFLAGS) -shared -o $@ oracle/ref_driver.c -L$(OUT) -lozl_ref -Wl,-rpath,'$$ORIGIN' -lm

.PHONY: all
