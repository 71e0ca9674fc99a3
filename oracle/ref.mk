# Builds oracle/_ref/libpmref.so: the reference's own photon-mapping code
# (photonMappingKernel.cu lines 6-1521) compiled as serial host C++ behind
# oracle/ref_shim.h. Test infrastructure: only tests/golden/make_golden.py
# loads it. Needs the reference checkout; outputs go to oracle/_ref/ only.
#
#   make -f oracle/ref.mk REF=<reference checkout>
ifndef REF
$(error REF=<path of the reference checkout> is required)
endif
OUT := oracle/_ref
CXX ?= g++

$(OUT)/libpmref.so: oracle/ref_harness.cpp oracle/ref_shim.h $(OUT)/ref_body.inc
	$(CXX) -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -w -fvisibility=hidden -Wl,-Bsymbolic \
	    -I oracle -I $(OUT) oracle/ref_harness.cpp -o $@

$(OUT)/ref_body.inc: $(REF)/photonMappingKernel.cu
	mkdir -p $(OUT)
	sed -n '6,1521p' "$<" > $@

.PHONY: clean
clean:
	rm -f $(OUT)/libpmref.so $(OUT)/ref_body.inc
