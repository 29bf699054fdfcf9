"""GB300-native engine for the tensor-product-basis sigma = H*C and Davidson."""
